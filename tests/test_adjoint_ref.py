"""The FP64 PyTorch re-implementation used to check the adjoint kernels is
itself checked here, on the CPU: its forward loss against the oracle's
field energy (the reference's algorithm), and its autograd gradients
against central finite differences."""
import math

import numpy as np
import pytest
import torch

from tests import adjoint_ref

L = 2 * math.pi


def _case(n, v0=0.2, amp=0.01):
    xt, y, sign, noise, uy = adjoint_ref.two_stream_state(n, L, v0, amp)
    return xt, y, sign, noise, uy


def test_forward_matches_oracle(orc):
    from oracle import oracle
    nx = ny = 32
    n, steps, dt = 2048, 40, 0.05
    q = -L * L / n
    xt, y, sign, noise, uy = _case(n)
    x, y, ux, uy = adjoint_ref.build_state(xt, y, sign, noise, uy, 0.2, 0.01, L)
    loss = adjoint_ref.field_energy(x, y, ux, uy, nx, ny, L, dt, 1.0, q, -q, steps).item()
    o = oracle.Oracle(nx, ny, L, L, dt, 1.0)
    o.add_species(q, -q, x.numpy(), y.numpy(), ux.numpy(), uy.numpy())
    o.pre_step()
    o.run(steps)
    o.stage_field_E()
    ex, ey = o.E()
    we = 0.5 * (L / nx) * (L / ny) * (np.sum(ex[:ny] ** 2) + np.sum(ey[:ny] ** 2))
    assert abs(loss - we) <= 1e-10 * we


def test_autograd_matches_finite_differences():
    nx = ny = 16
    n, steps, dt = 512, 30, 0.05
    q = -L * L / n
    xt, y, sign, noise, uy = _case(n)

    def loss_of(v0, amp):
        x, yy, ux, uyy = adjoint_ref.build_state(xt, y, sign, noise, uy, v0, amp, L)
        return adjoint_ref.field_energy(x, yy, ux, uyy, nx, ny, L, dt, 1.0, q, -q, steps)

    v0 = torch.tensor(0.2, dtype=torch.float64, requires_grad=True)
    amp = torch.tensor(0.01, dtype=torch.float64, requires_grad=True)
    loss_of(v0, amp).backward()
    eps = 1e-6
    with torch.no_grad():
        fd_v0 = (loss_of(0.2 + eps, 0.01) - loss_of(0.2 - eps, 0.01)).item() / (2 * eps)
        fd_amp = (loss_of(0.2, 0.01 + eps) - loss_of(0.2, 0.01 - eps)).item() / (2 * eps)
    assert abs(v0.grad.item() - fd_v0) <= 1e-5 * abs(fd_v0)
    assert abs(amp.grad.item() - fd_amp) <= 1e-5 * abs(fd_amp)
