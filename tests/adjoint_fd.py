"""Finite differences of the adjoint workload's loss with the cell-edge
crossings accounted for.

The CIC weights are piecewise linear in the position, so the field energy
after N steps has a kink wherever a particle's trajectory puts it on a cell
edge.  A central difference L(p + eps d) - L(p - eps d) over a direction d
picks up a term from every particle whose cell sequence differs between the
two perturbed runs (it "straddles" an edge): such a difference is not the
derivative, whatever the adjoint computes.  So:

- straddlers(): runs the FP64 step from the two perturbed initial states in
  lockstep and marks every particle whose cell differs between the runs at
  any step (positions compared after every step, iteration 0 included);
- the perturbation is then restricted to the particles that do not
  straddle, the check is repeated on the restricted runs (a particle can
  still straddle through the change of the field), and the central
  difference along the restricted direction is compared with the adjoint's
  gradient projected on the same direction;
- what straddles through the field leaves a kink term of first order in
  eps (a number of straddlers proportional to eps, each off by an amount
  proportional to eps, over 2 eps), while the smooth part's error is second
  order: the Richardson combination 2 D(eps/2) - D(eps) removes it.

Test and study infrastructure (tests/test_gpu_adjoint.py, bench.py --study
adjoint).
"""
import math

import numpy as np

from cpic_gb300 import _lib


def _cells(ctx, grid, L):
    x, y, _, _ = ctx.particles(0)
    dx = L / grid
    return (np.floor(y / dx).astype(np.int64) * grid + np.floor(x / dx).astype(np.int64))


def straddlers(grid, L, dt, q, s_plus, s_minus, steps):
    """Boolean mask of the particles whose cell differs between the runs
    from the states s_plus and s_minus ((x, y, ux, uy) arrays) at any of
    the `steps` steps (and at the start)."""
    ctx = []
    for st in (s_plus, s_minus):
        c = _lib.Context(grid, grid, L, L, dt, 1.0, precision=_lib.FP64, track_ids=True)
        c.add_species(q, -q, *st)
        c.pre_step()
        ctx.append(c)
    mask = _cells(ctx[0], grid, L) != _cells(ctx[1], grid, L)
    for _ in range(steps):
        for c in ctx:
            c.step()
        mask |= _cells(ctx[0], grid, L) != _cells(ctx[1], grid, L)
    for c in ctx:
        c.close()
    return mask


def restricted_fd(adj, grid, L, dt, q, steps, base, direction, grad, eps, rounds=2):
    """Central difference of the loss along `direction` (per-array
    perturbations of base = (x, y, ux, uy)) restricted to the particles that
    straddle no cell edge, against the adjoint gradient `grad` projected on
    the same direction.  Returns a dict with the straddler fractions of the
    full and of the restricted perturbation, the difference quotient, the
    projected gradient and their relative difference."""
    n = len(base[0])
    keep = np.ones(n, bool)
    out = {"eps": eps}

    def perturbed(step, m):
        s = [a.copy() for a in base]
        for k, d in enumerate(direction):
            if d is not None:
                s[k] = s[k] + step * d * m
        s[0] = np.mod(s[0], L)
        return s

    for r in range(rounds):
        m = keep.astype(np.float64)
        sp, sm = perturbed(eps, m), perturbed(-eps, m)
        strad = straddlers(grid, L, dt, q, sp, sm, steps)
        out["straddle_fraction_round%d" % r] = float(strad.mean())
        if r == 0:
            out["straddle_fraction_full"] = float(strad.mean())
        if r + 1 < rounds:
            keep &= ~strad
        else:
            out["straddlers_left"] = int(strad.sum())
    m = keep.astype(np.float64)

    def quotient(e):
        return (adj.forward(*perturbed(e, m)) - adj.forward(*perturbed(-e, m))) / (2 * e)

    fd = quotient(eps)
    # the kink term of the particles that still straddle (through the field)
    # is first order in eps, unlike the smooth part's second-order error:
    # the Richardson combination of eps and eps/2 cancels it
    fd_half = quotient(eps / 2)
    rich = 2.0 * fd_half - fd
    proj = float(sum(np.sum(g * d * m) for g, d in zip(grad, direction) if d is not None))
    out.update({"fd": fd, "fd_half_eps": fd_half, "fd_richardson": rich, "adjoint": proj,
                "rel_diff": abs(fd - proj) / abs(proj),
                "rel_diff_richardson": abs(rich - proj) / abs(proj),
                "particles_perturbed": int(keep.sum())})
    return out


def two_stream_directions(xt, sign, L):
    """Per-array directions of d/dv0 (ux += sign) and d/damp
    (x += sin(2 pi xt / L)) of the two-stream state."""
    return ((None, None, sign, None), (np.sin(2 * math.pi * xt / L), None, None, None))
