"""FP64 PyTorch re-implementation of the step, differentiated by autograd:
the independent check of the hand-written adjoint kernels.

TEST INFRASTRUCTURE.  The same step as the library's adjoint run (and the
reference's algorithm, sim.c:481-581): CIC deposit with -q/e0 per unit
weight (interpolate.c:282-346), periodic FFT Poisson with the reference's
Green's function (solver.c:257-280, 465-509), E by periodic central
differences (field.c:358-416), CIC gather (interpolate.c:349-404), Boris
for B along z (mover.c:15-92) with the iteration-0 backward half kick and
no move (mover.c:204-213), periodic wrap (comm_plasma.c:726-747).  Loss:
1/2 e0 dx dy sum |E|^2 of the field solved from the final positions.
"""
import math

import torch


def _weights(x, y, nx, ny, dx, dy):
    gx, gy = x / dx, y / dy
    fx0, fy0 = torch.floor(gx).detach(), torch.floor(gy).detach()
    fx, fy = gx - fx0, gy - fy0
    ix = fx0.long() % nx
    iy = fy0.long() % ny
    ix1, iy1 = (ix + 1) % nx, (iy + 1) % ny
    idx = [iy * nx + ix, iy * nx + ix1, iy1 * nx + ix, iy1 * nx + ix1]
    w = [(1 - fx) * (1 - fy), fx * (1 - fy), (1 - fx) * fy, fx * fy]
    return idx, w


def field_energy(x, y, ux, uy, nx, ny, L, dt, e0, q, m, nsteps, Bz=0.0):
    """Differentiable loss of the initial state (FP64 tensors)."""
    dev, dt_ = x.device, torch.float64
    dx, dy = L / nx, L / ny
    kx = torch.arange(nx // 2 + 1, dtype=dt_, device=dev)
    ky = torch.arange(ny, dtype=dt_, device=dev)
    G = 1.0 / (2.0 * (torch.cos(2 * math.pi * kx / nx)[None, :]
                      + torch.cos(2 * math.pi * ky / ny)[:, None]) - 4.0)
    G[0, 0] = 0.0
    c = -q / e0

    def field(px, py):
        idx, w = _weights(px, py, nx, ny, dx, dy)
        rho = torch.zeros(nx * ny, dtype=dt_, device=dev)
        for i, ww in zip(idx, w):
            rho = rho.index_add(0, i, ww * c)
        rho = rho.reshape(ny, nx)
        phi = torch.fft.irfft2(G * torch.fft.rfft2(rho), s=(ny, nx))
        Ex = (torch.roll(phi, 1, dims=1) - torch.roll(phi, -1, dims=1)) / (2 * dx)
        Ey = (torch.roll(phi, 1, dims=0) - torch.roll(phi, -1, dims=0)) / (2 * dy)
        return Ex.reshape(-1), Ey.reshape(-1)

    for j in range(nsteps):
        Ex, Ey = field(x, y)
        idx, w = _weights(x, y, nx, ny, dx, dy)
        ex = sum(ww * Ex[i] for i, ww in zip(idx, w))
        ey = sum(ww * Ey[i] for i, ww in zip(idx, w))
        dtp = -0.5 * dt if j == 0 else dt
        h = 0.5 * dtp * q / m
        t = Bz * h
        s = 2 * t / (1 + t * t)
        vmx, vmy = ux + h * ex, uy + h * ey
        vpx, vpy = vmx + vmy * t, vmy - vmx * t
        ux = vmx + vpy * s + h * ex
        uy = vmy - vpx * s + h * ey
        if j > 0:
            x = torch.remainder(x + dt * ux, L)
            y = torch.remainder(y + dt * uy, L)
    Ex, Ey = field(x, y)
    return 0.5 * e0 * dx * dy * (Ex.square().sum() + Ey.square().sum())


def two_stream_state(n, L, v0, amp, seed=7, vth=0.0):
    """Initial state as torch tensors: (x~, y, sign) with x = x~ + amp
    sin(2 pi x~ / L) wrapped and ux = sign v0 (+ vth noise)."""
    from cpic_gb300 import _lib
    xt, y, ux, uy = _lib.init_two_stream(seed, 0, n, L, L, 1.0, vth, 0.0)
    sign = torch.where(torch.arange(n) < n // 2, 1.0, -1.0).double()
    noise = torch.from_numpy(ux).double() - sign
    return torch.from_numpy(xt), torch.from_numpy(y), sign, noise, torch.from_numpy(uy)


def build_state(xt, y, sign, noise, uy, v0, amp, L):
    """Differentiable map (v0, amp) -> initial particle state."""
    x = torch.remainder(xt + amp * torch.sin(2 * math.pi * xt / L), L)
    ux = sign * v0 + noise
    return x, y, ux, uy
