"""The integer forms of the FP64 form's conversions (cpic_gb300/csrc/cpic_bits.h:
floor to the cell index, and the fixed-point split of a deposit value into
rn(v) and rn((v - rn(v)) 2^m)) give the FP64 instructions' results bit for
bit: edge cases (exact ties at many scales, their neighbours, zeros, values
near 2^31) and 8 million random values of both signs over 2^-320 .. 2^60.
CPU only: the same header is compiled for the device."""
import os
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))


def test_integer_conversions_match_fp64():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "bits_check")
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "bits_check.cpp"),
                        "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-3000:]
    assert r.stdout.strip().startswith("0 mismatches"), r.stdout
