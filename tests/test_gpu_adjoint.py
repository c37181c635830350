"""Adjoint run on the GPU (cpic_adj_*): gradient of the final field energy
with respect to the initial state.

- its forward pass is the step: the loss equals the FP64 step's field
  energy after the same steps;
- gradients for every particle against an independent FP64 PyTorch
  re-implementation differentiated by autograd (tests/adjoint_ref.py, itself
  pinned to the oracle and to finite differences on the CPU), on 1/64 of
  the adjoint workload (128x128, 16,384 electrons, 200 steps, checkpoint
  every 20); also through the torch.autograd binding;
- dL/dv0, dL/damp and single-particle dL/du on the full adjoint workload
  (1,048,576 electrons) against FP64 central finite differences (eps 1e-6
  as prescribed, and 1e-8 / 1e-9 where the CIC kink term is smaller);
- the FP32 adjoint against the same finite differences;
- checkpoint interval does not change the result (recompute is exact);
- cost of the backward sweep against the forward run.
"""
import math

import numpy as np
import pytest
import torch

from cpic_gb300 import _lib
from cpic_gb300.autograd import field_energy
from tests import adjoint_ref

pytestmark = pytest.mark.gpu
L = 2 * math.pi


def _adj(n, grid, steps, K, prec=_lib.FP64):
    q = -L * L / n
    return _lib.Adjoint(grid, grid, L, L, 0.05, 1.0, q, -q, n, steps, K, precision=prec)


def _state(n, v0=0.2, amp=0.01, seed=7):
    xt, y, sign, noise, uy = adjoint_ref.two_stream_state(n, L, v0, amp, seed=seed)
    return xt, y, sign, noise, uy


def _np_state(st, v0, amp):
    return [t.numpy() for t in adjoint_ref.build_state(*st, v0, amp, L)]


def _chain(st, g):
    """dL/dv0 and dL/damp from the per-particle gradient."""
    xt, _, sign, _, _ = st
    return (float(np.sum(sign.numpy() * g[2])),
            float(np.sum(np.sin(2 * math.pi * xt.numpy() / L) * g[0])))


def test_forward_is_the_step(lib):
    n, grid, steps = 10240, 64, 50
    st = _state(n)
    x, y, ux, uy = _np_state(st, 0.2, 0.01)
    adj = _adj(n, grid, steps, 10)
    loss = adj.forward(x, y, ux, uy)
    q = -L * L / n
    c = _lib.Context(grid, grid, L, L, 0.05, 1.0, precision=_lib.FP64)
    c.add_species(q, -q, x, y, ux, uy)
    c.pre_step()
    c.run(steps)
    c.stage_field_E()
    ref = c.field_energy()
    assert abs(loss - ref) <= 1e-12 * ref


def test_gradient_matches_torch_autograd(lib):
    n, grid, steps = 16384, 128, 200
    st = _state(n)
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    leaves = [t.to(dev).requires_grad_(True) for t in adjoint_ref.build_state(*st, 0.2, 0.01, L)]
    q = -L * L / n
    lt = adjoint_ref.field_energy(*leaves, grid, grid, L, 0.05, 1.0, q, -q, steps)
    lt.backward()
    tg = [t.grad.cpu().numpy() for t in leaves]
    adj = _adj(n, grid, steps, 20)
    loss = adj.forward(*[t.detach().cpu().numpy() for t in leaves])
    g = adj.backward()
    assert abs(loss - lt.item()) <= 1e-10 * lt.item()
    for a, b in zip(g, tg):
        assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(b)
    ours, theirs = _chain(st, g), _chain(st, tg)
    for a, b in zip(ours, theirs):
        assert abs(a - b) <= 1e-6 * abs(b)
    # the torch.autograd binding: gradients flow back to v0 and amp
    v0 = torch.tensor(0.2, dtype=torch.float64, requires_grad=True)
    amp = torch.tensor(0.01, dtype=torch.float64, requires_grad=True)
    x, y, ux, uy = adjoint_ref.build_state(*st, v0, amp, L)
    field_energy(adj, x, y, ux, uy).backward()
    assert abs(v0.grad.item() - theirs[0]) <= 1e-6 * abs(theirs[0])
    assert abs(amp.grad.item() - theirs[1]) <= 1e-6 * abs(theirs[1])


def test_checkpoint_interval_does_not_change_gradients(lib):
    n, grid, steps = 4096, 32, 30
    st = _state(n)
    s = _np_state(st, 0.2, 0.01)
    out = []
    for K in (1, 7, 30):
        adj = _adj(n, grid, steps, K)
        adj.forward(*s)
        out.append(adj.backward())
    for g in out[1:]:
        for a, b in zip(g, out[0]):
            assert np.array_equal(a, b)


@pytest.fixture(scope="module")
def c5():
    """The adjoint workload: 128x128, 64 electrons per cell (1,048,576),
    v0 0.2, amplitude 0.01, 200 steps, checkpoint every 20, with FP64
    central differences of the loss in v0 and amp at eps 1e-6, 1e-8, 1e-9."""
    n, grid, steps, K = 128 * 128 * 64, 128, 200, 20
    st = _state(n, seed=11)
    adj = _adj(n, grid, steps, K)
    f = lambda v0, amp: adj.forward(*_np_state(st, v0, amp))
    fd = {}
    for eps in (1e-6, 1e-8, 1e-9):
        fd[eps] = ((f(0.2 + eps, 0.01) - f(0.2 - eps, 0.01)) / (2 * eps),
                   (f(0.2, 0.01 + eps) - f(0.2, 0.01 - eps)) / (2 * eps))
    return dict(n=n, grid=grid, steps=steps, K=K, st=st, adj=adj, fd=fd)


def _rel(a, b):
    return abs(a - b) / abs(b)


def test_fp64_gradient_matches_finite_differences(lib, c5):
    """CIC weights are piecewise linear: the loss has a kink wherever a
    particle crosses a cell edge, and over 200 steps a v0 step of 1e-6 moves
    enough of the million particles across edges that the central
    difference carries ~5e-4 of truncation from the kinks (measured:
    6e-3, 4e-4, 5e-4, 2e-4, 1e-4, 1.5e-5 for eps 1e-4 ... 1e-9).  So: within
    1e-3 at the prescribed eps 1e-6, and within 1e-4 at eps 1e-8 or 1e-9,
    where the kink term has shrunk and rounding has not yet grown."""
    adj, st = c5["adj"], c5["st"]
    base = _np_state(st, 0.2, 0.01)
    adj.forward(*base)
    g = adj.backward()
    dv0, damp = _chain(st, g)
    fd = c5["fd"]
    assert _rel(dv0, fd[1e-6][0]) <= 1e-3 and _rel(damp, fd[1e-6][1]) <= 1e-3
    assert min(_rel(dv0, fd[e][0]) for e in (1e-8, 1e-9)) <= 1e-4
    assert min(_rel(damp, fd[e][1]) for e in (1e-8, 1e-9)) <= 1e-4
    # single initial velocities: the kink term is small, eps 1e-6
    eps = 1e-6
    for i in (0, 777777):
        for comp in (2, 3):
            p = [a.copy() for a in base]
            p[comp][i] += eps
            lp = adj.forward(*p)
            p[comp][i] -= 2 * eps
            lm = adj.forward(*p)
            fdi = (lp - lm) / (2 * eps)
            assert abs(g[comp][i] - fdi) <= 1e-3 * abs(fdi) + 1e-12, (i, comp, g[comp][i], fdi)


def test_fp32_gradient_against_fp64_finite_differences(lib, c5):
    st = c5["st"]
    adj = _adj(c5["n"], c5["grid"], c5["steps"], c5["K"], _lib.MIXED)
    adj.forward(*_np_state(st, 0.2, 0.01))
    dv0, damp = _chain(st, adj.backward())
    fd = c5["fd"][1e-8]
    assert _rel(dv0, fd[0]) <= 2e-3 and _rel(damp, fd[1]) <= 2e-3


def test_backward_cost(lib, c5):
    adj, st = c5["adj"], c5["st"]
    adj.forward(*_np_state(st, 0.2, 0.01))
    adj.backward()
    tf, tb = adj.times()
    assert tb <= 3.0 * tf, (tf, tb)


def test_fd_at_prescribed_eps_with_edge_crossings_accounted(lib, c5):
    """At the prescribed eps 1e-6 the plain central difference is off by the
    kink term of the particles that cross a cell edge differently in the
    two perturbed runs (tests/adjoint_fd.py).  Restricting the perturbation
    to the particles that straddle no edge removes the direct part of that
    term.  For v0, where most straddlers are perturbed directly, the
    difference quotient along the restricted direction then matches the
    adjoint's gradient projected on it within 1e-4, and the Richardson
    combination of eps 1e-6 and 5e-7 within 1e-5.  For the amplitude, the
    straddlers are mostly particles whose own state is not perturbed (they
    cross through the change of the field), so restricting the direction
    cannot remove them; the bound there documents what is left."""
    from tests import adjoint_fd
    adj, st = c5["adj"], c5["st"]
    base = _np_state(st, 0.2, 0.01)
    adj.forward(*base)
    g = adj.backward()
    q = -L * L / c5["n"]
    xt, _, sign, _, _ = st
    dirs = adjoint_fd.two_stream_directions(xt.numpy(), sign.numpy(), L)
    for name, d in zip(("v0", "amp"), dirs):
        r = adjoint_fd.restricted_fd(adj, c5["grid"], L, 0.05, q, c5["steps"], base, d, g, 1e-6)
        print(name, r)
        assert 0.0 < r["straddle_fraction_full"] < 0.5
        if name == "v0":
            # 4.1 % of the particles straddle; restricted: 7.5e-5, and the
            # Richardson combination 3.8e-6 (measured)
            assert r["rel_diff"] <= 1e-4 and r["rel_diff_richardson"] <= 1e-5, (name, r)
        else:
            # 0.70 % straddle, 0.64 % of them through the change of the field
            # (their own initial state is not perturbed): what is left is the
            # kink term of those, 1.2e-4 measured, not first order in eps
            # (Richardson gives 2.3e-4).  At eps 1e-8, where it has shrunk,
            # the amplitude gradient agrees to 3.3e-6 (the test above).
            assert r["straddlers_left"] > 0.8 * r["straddle_fraction_full"] * c5["n"]
            assert r["rel_diff"] <= 2e-4, (name, r)
