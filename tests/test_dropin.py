"""The drop-in sim layer (cpic_gb300/dropin/sim_gpu.c) against the
reference's own callers: src/cpic.c and test/{constant-speed,cyclotron,harmonic}.c
link unchanged against it and libcpic_gb300, with sim_init / sim_step /
sim_run resolved from the drop-in.  Without a GPU, running them goes
through the reference's whole host initialisation (config, species,
fields, plasma, init method) and stops cleanly at cpic_create."""
import os
import subprocess

import pytest

from tests import dropin_build

pytestmark = pytest.mark.skipif(not os.path.isdir(dropin_build.REF),
                                reason="needs the reference tree")


@pytest.fixture(scope="module")
def out(lib):
    d = dropin_build.build()
    if d is None:
        pytest.skip("reference host objects are x86-64 only")
    return d


def test_sim_entry_points_come_from_dropin(out):
    syms = subprocess.run(["nm", os.path.join(out, "sim_gpu.o")], capture_output=True,
                          text=True, check=True).stdout
    defined = {l.split()[-1] for l in syms.splitlines() if " T " in l}
    assert {"sim_init", "sim_step", "sim_run"} <= defined
    undefined = {l.split()[-1] for l in syms.splitlines() if " U " in l}
    # the hot path comes from the GPU library, not from the reference
    assert not undefined & {"stage_field_E", "stage_plasma_E", "stage_plasma_r",
                            "stage_field_rho", "comm_plasma", "solver_init", "solve_xy"}
    assert {"cpic_create", "cpic_pre_step", "cpic_step", "cpic_stage_plasma"} <= undefined


CONF = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "cpic_gb300",
                    "dropin", "conf", "two_stream_64.conf")


@pytest.mark.parametrize("prog,conf", [("test_constant_speed_gpu", None),
                                       ("test_cyclotron_gpu", None),
                                       ("test_harmonic_gpu", None),
                                       ("cpic_gpu", "conf/constant-speed.conf"),
                                       ("cpic_gpu", CONF)])
def test_reference_callers_reach_gpu_library(out, prog, conf):
    import torch
    if torch.cuda.is_available():
        pytest.skip("with a GPU these run for real; this test covers the host path")
    cmd = [os.path.join(out, prog)] + ([conf] if conf else [])
    r = subprocess.run(cmd, cwd=dropin_build.REF, capture_output=True, text=True, timeout=120)
    assert r.returncode != 0
    assert "sim_gpu: cpic_create failed with status -8" in r.stderr, r.stderr
    assert "missing parameter" not in r.stderr
