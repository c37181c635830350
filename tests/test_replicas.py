"""bench.py under torch.distributed.run with two ranks on the CPU (gloo):
the reference arm runs on rank 0 alone and prints one JSON line, the other
rank exits 0 without work; the max-over-ranks timing helper reduces over
both ranks."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout=240):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", "--master-port=%d" % _port()] + args
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=timeout, env=env)


def test_reference_arm_two_ranks(lib, orc):
    r = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
                   "--workload", "two_stream_64"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["n_gpus"] == 2 and out["value"] > 0
    # the reference's own build where it is built here, else its restatement
    from oracle import ref_run
    kind = "reference" if ref_run.harness() else "port"
    assert out["e2e"]["h2d_bytes_per_step"] == 0 and out["cpu_baseline"]["kind"] == kind


def test_max_over_ranks_gloo(tmp_path):
    out = tmp_path / "rank"
    script = ("import os, sys; sys.path.insert(0, %r); import bench, torch.distributed as td; "
              "td.init_process_group('gloo'); r = int(os.environ['RANK']); "
              "v = bench.max_over_ranks(1.0 + r); bench.barrier(); "
              "open(%r + str(r), 'w').write(repr(v)); td.destroy_process_group()" % (ROOT, str(out)))
    path = tmp_path / "replica_probe.py"
    path.write_text(script.replace("; ", "\n"))
    r = _torchrun([str(path)])
    assert r.returncode == 0, r.stderr[-2000:]
    assert [(tmp_path / ("rank%d" % k)).read_text() for k in (0, 1)] == ["2.0", "2.0"]


def test_reference_arm_skips_grids_not_power_of_two():
    """On a grid whose side is not a power of two the FFTW stand-in the
    reference is built against here is far slower than FFTW: the reference
    arm prints its unavailable line at once instead of a flattering time."""
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--workload", "two_stream_1920"],
                       cwd=ROOT, capture_output=True, text=True, timeout=120,
                       env=dict(os.environ, CUDA_VISIBLE_DEVICES=""))
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][0])
    assert out["impl"] == "reference" and "not a power of two" in out["unavailable"]
