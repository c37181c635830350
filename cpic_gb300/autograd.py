"""torch.autograd binding of the adjoint run (cpic_adj_* in
include/cpic_gpu.h): a thin test binding, the kernels are the library's.

    adj = _lib.Adjoint(nx, ny, Lx, Ly, dt, e0, q, m, n, nsteps, K)
    loss = field_energy(adj, x, y, ux, uy)     # tensors of n particles
    loss.backward()                            # x.grad ... from the adjoint

Any torch expression may produce x, y, ux, uy (e.g. a beam speed and a
perturbation amplitude that require grad); autograd chains through it.
"""
import torch


class FieldEnergy(torch.autograd.Function):
    """L = 1/2 e0 dx dy sum |E|^2 after adj's nsteps, as a function of the
    initial positions and velocities."""

    @staticmethod
    def forward(ctx, adj, x, y, ux, uy):
        host = [t.detach().to("cpu", torch.float64).numpy() for t in (x, y, ux, uy)]
        loss = adj.forward(*host)
        ctx.adj = adj
        ctx.device = x.device
        return torch.tensor(loss, dtype=torch.float64, device=x.device)

    @staticmethod
    def backward(ctx, g):
        grads = ctx.adj.backward()
        out = [g * torch.from_numpy(a).to(ctx.device) for a in grads]
        return (None, *out)


def field_energy(adj, x, y, ux, uy):
    return FieldEnergy.apply(adj, x, y, ux, uy)
