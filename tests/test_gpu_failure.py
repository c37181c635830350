"""Failure paths on the GPU, made on the host or by a wait that nothing
completes; no test faults, traps or hangs the device.

- The reference aborts when a particle's speed exceeds umax = chunksize dx / dt
  (src/mover.c:97-137, src/sim.c:198-200).  Here the push records a status
  bit and the step returns CPIC_EUMAX; the context stays usable and
  destroyable.  The state is injected on the host: one particle of a
  two-stream plasma gets ux above umax.
- Every wait of the library's shared-memory pipeline is bounded.  The
  self-test entry point makes one such wait run out on an mbarrier phase that
  no copy completes (none is issued) and must report CPIC_ETIMEOUT; the
  device then runs a fresh context normally.
"""
import pytest

from cpic_gb300 import _lib
from oracle.oracle import Oracle
from tests import cases

pytestmark = pytest.mark.gpu


def fast_particle_case(chunks):
    case = cases.two_stream(n=10240)
    dx = case["L"] / case["nx"]
    umax = (case["nx"] // chunks) * dx / case["dt"]
    case["species"][0]["ux"] = case["species"][0]["ux"].copy()
    case["species"][0]["ux"][17] = 1.5 * umax
    return case, umax


@pytest.mark.parametrize("precision", [_lib.FP64, _lib.MIXED])
def test_velocity_above_umax_returns_eumax(lib, precision):
    chunks = 64                        # one cell per chunk: umax = dx / dt
    case, umax = fast_particle_case(chunks)
    L = case["L"]
    ctx = _lib.Context(case["nx"], case["ny"], L, L, case["dt"], 1.0, case["B"], precision=precision,
                       plasma_chunks=chunks)
    s = case["species"][0]
    ctx.add_species(s["q"], s["m"], s["x"], s["y"], s["ux"], s["uy"])
    ctx.pre_step()
    with pytest.raises(_lib.CpicError) as err:
        ctx.step()
    assert err.value.code == -4        # CPIC_EUMAX
    ctx.close()
    # the oracle (the reference's algorithm) stops on the same state
    o = Oracle(case["nx"], case["ny"], L, L, case["dt"], 1.0, case["B"], plasma_chunks=chunks)
    o.add_species(s["q"], s["m"], s["x"], s["y"], s["ux"], s["uy"])
    o.pre_step()
    with pytest.raises(RuntimeError):
        o.step()
    o.close()
    # below umax nothing is reported
    case["species"][0]["ux"][17] = 0.9 * umax
    ok = _lib.Context(case["nx"], case["ny"], L, L, case["dt"], 1.0, case["B"], precision=precision,
                      plasma_chunks=chunks)
    ok.add_species(s["q"], s["m"], s["x"], s["y"], s["ux"], s["uy"])
    ok.pre_step()
    ok.step()
    ok.step()
    ok.close()


def test_bounded_wait_expires_and_device_stays_usable(lib):
    assert lib.cpic_selftest_wait(64) == -10     # CPIC_ETIMEOUT
    assert lib.cpic_selftest_wait(0) == -1
    assert lib.cpic_selftest_wait(1 << 21) == -1
    case = cases.two_stream(n=4096)
    g = cases.make_gpu(case)
    o = cases.make_oracle(case)
    g.pre_step()
    o.pre_step()
    for _ in range(3):
        g.step()
        o.step()
        we_g, we_o = g.diag()["WE"], o.diag()["WE"]
        assert abs(we_g - we_o) <= 1e-10 * we_o
    g.close()
