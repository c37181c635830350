"""cpic_poisson_noalloc: the Poisson solve for callers that cannot allocate
device memory (a fixed memory budget or their own pool owning the device, or
threads on which cudaMalloc/cudaFree and their implicit synchronisation must
not appear).  Its scratch is a static device array shared by every call, so
the test calls it twice in a row with different inputs and checks each
result against the context's field stage (cpic_set_rho, cpic_stage_field_E,
cpic_get_phi) and against the oracle's FP64 Poisson solve, within the 1e-12
relative tolerance used for phi elsewhere.  The caller (this test) owns the
input and output device buffers.

Kept in its own file, collected last, so that a run stopping at the first
failure has already run every other test; it also passes alone in a fresh
process (the first call looks up the array's device address)."""
import numpy as np
import pytest

from cpic_gb300 import _lib
from oracle import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-12


def field_stage_phi(rho):
    ny, nx = rho.shape
    ctx = _lib.Context(nx, ny, 1.0, 1.0, 0.1, precision=_lib.FP64)
    # one heavy particle only fixes the fixed-point charge scale (range +-2^11)
    ctx.add_species(1e3, 1.0, [0.5], [0.5], [0.0], [0.0])
    ctx.set_rho(rho)
    ctx.stage_field_E()
    phi = ctx.phi()
    ctx.close()
    return phi


@pytest.mark.parametrize("nx,ny", [(4, 4), (64, 32), (512, 512)])
def test_noalloc_matches_field_stage_twice(lib, nx, ny):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(nx * 7 + ny)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        rho = rng.standard_normal((ny, nx))
        d_rho = torch.from_numpy(rho).cuda()
        d_phi = torch.full_like(d_rho, float("nan"))
        r = lib.cpic_poisson_noalloc(d_rho.data_ptr(), d_phi.data_ptr(), nx, ny, stream)
        assert r == 0, r
        torch.cuda.synchronize()
        got = d_phi.cpu().numpy()
        want = field_stage_phi(rho)
        rel = np.max(np.abs(got - want)) / np.max(np.abs(want))
        assert rel <= TOL, (call, rel)
        ref = oracle.poisson(rho)
        rel = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert rel <= TOL, (call, rel)


def test_noalloc_rejects_grids_beyond_its_array(lib):
    torch = pytest.importorskip("torch")
    big = torch.zeros((1024, 1024), dtype=torch.float64, device="cuda")
    assert lib.cpic_poisson_noalloc(big.data_ptr(), big.data_ptr(), 1024, 1024, None) == -1
    assert lib.cpic_poisson_noalloc(big.data_ptr(), big.data_ptr(), 48, 32, None) == -1


def test_fp64_field_stage_after_noalloc(lib):
    """The no-allocation solve has its own copies of the FFT kernels: calling
    it first leaves the contexts' kernels, and their shared-memory limits,
    alone.  A 4096-wide FP64 grid needs 128 KB of shared memory per row
    block of the context's solve."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    rho = rng.standard_normal((32, 32))
    d_rho = torch.from_numpy(rho).cuda()
    d_phi = torch.empty_like(d_rho)
    assert lib.cpic_poisson_noalloc(d_rho.data_ptr(), d_phi.data_ptr(), 32, 32, None) == 0
    torch.cuda.synchronize()
    wide = rng.standard_normal((64, 4096))
    got = field_stage_phi(wide)
    ref = oracle.poisson(wide)
    assert np.max(np.abs(got - ref)) <= TOL * np.max(np.abs(ref))
