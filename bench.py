"""Benchmark: particle-steps/s of the 2D electrostatic PIC step on one GB300.

Workload (default): two-stream instability on a periodic 2048x2048 grid,
L = 2 pi, 100 electrons per cell (419,430,400 particles), beams +-0.2 with
Maxwellian spread 0.01 and a 0.01 sinusoidal perturbation in x, dt = 0.05,
mixed precision (int32 cell + FP32 offset, FP32 velocity and E, FP64
charge reduction and diagnostics).  Synthetic inputs from the library's
seeded init method.  The FP64 plain form runs the same workload for the
speed-up and the field-energy error.

One JSON line on rank 0.  `value` is device-resident throughput timed with
CUDA events; `e2e` goes through the C ABI from host buffers over the
workload's whole run of 1000 steps (upload, pre-step, the steps with a
per-step field-energy read-back, download).
`--impl reference` times the oracle (the CPU restatement of the reference's
FP64 step) on the host cores instead.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300: FP32-offset vs FP64 plain at ≤1e-5 rel field-energy err"
UNIT = "particle-steps/s"
B_P = {"mixed": 40.0, "fp64": 64.0}     # algorithmic bytes per particle-step
B_G = {"mixed": 40.0, "fp64": 48.0}     # algorithmic bytes per grid node per step
KERNELS_PER_STEP = 7                     # the benchmark workload has one species

WORKLOADS = {
    # name: (grid, particles per cell, v0, vth, amp, description)
    "two_stream_2048": (2048, 100, 0.2, 0.01, 0.01,
                        "two-stream 2048x2048, 100 electrons/cell (419,430,400), beams +-0.2, "
                        "vth 0.01, amp 0.01, dt 0.05"),
    "two_stream_1024": (1024, 100, 0.2, 0.01, 0.01,
                        "two-stream 1024x1024, 100 electrons/cell (104,857,600), beams +-0.2, "
                        "vth 0.01, amp 0.01, dt 0.05"),
    "two_stream_512": (512, 100, 0.2, 0.01, 0.01,
                       "two-stream 512x512, 100 electrons/cell (26,214,400), beams +-0.2, vth 0.01, "
                       "amp 0.01, dt 0.05"),
    "two_stream_64": (64, 100, 0.2, 0.01, 0.01, "two-stream 64x64, 100 electrons/cell (409,600)"),
    # a grid whose side is not a power of two (1920 = 2^7 3 5: mixed-radix field
    # solve, compare-wrapped cells) with the benchmark's 32x32 tiles
    "two_stream_1920": (1920, 100, 0.2, 0.01, 0.01,
                        "two-stream 1920x1920, 100 electrons/cell (368,640,000), beams +-0.2, "
                        "vth 0.01, amp 0.01, dt 0.05"),
}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0}, "fallback"


def profile_value(key):
    """A per-particle figure of the fused particle kernel from the committed
    ncu summary (profiles/k_push_traffic.txt, `key: value` lines), or None."""
    path = os.path.join(ROOT, "profiles", "k_push_traffic.txt")
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return float(line.split(":")[1])
    except (OSError, ValueError):
        pass
    return None


def profile_traffic(form):
    """DRAM bytes per particle of the fused particle kernel, or None."""
    return profile_value("traffic_bytes_per_particle_%s" % form)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []          # (host time, fields)
        self.proc = None
        self.t0 = self.t1 = None

    def start(self):
        """Starts sampling every 20 ms and waits (up to 5 s) for the first
        reading, so that the sampler is live when the timed region starts."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t_end = time.perf_counter() + 5.0
            while not self.samples and time.perf_counter() < t_end:
                time.sleep(0.005)
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append((time.perf_counter(), parts))

    def mark_start(self):
        self.t0 = time.perf_counter()

    def mark_end(self):
        self.t1 = time.perf_counter()

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        # readings taken inside the timed region (host clock); if the region
        # was shorter than the sampling interval, the first reading after
        # its start
        inside = [p for t, p in self.samples
                  if self.t0 is not None and self.t0 <= t <= (self.t1 or t)]
        if not inside:
            after = [p for t, p in self.samples if self.t0 is None or t >= self.t0]
            inside = after[:1]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for p in inside:
            try:
                sm.append(float(p[0]))
                mx = float(p[1])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if p[3 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm),
                "window_s": round(self.t1 - self.t0, 4) if self.t0 and self.t1 else None}


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def barrier():
    ws, _ = dist()
    if ws > 1:
        import torch.distributed as td
        td.barrier()


def max_over_ranks(v):
    ws, _ = dist()
    if ws == 1:
        return v
    import torch
    import torch.distributed as td
    t = torch.tensor([v], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def make_state(grid, ppc, v0, vth, amp, seed=2024):
    from cpic_gb300 import _lib
    n = grid * grid * ppc
    L = 2 * math.pi
    x, y, ux, uy = _lib.init_two_stream(seed, 0, n, L, L, v0, vth, amp)
    q = -L * L / n
    return dict(n=n, L=L, q=q, m=-q, x=x, y=y, ux=ux, uy=uy)


TILE = {"tile": 0, "halo": 0}
DATA = "synthetic (seeded two-stream init, SplitMix64)"


def bench_config(grid, ppc, desc):
    """The workload's config, identical in both arms (precision goes in
    dtype)."""
    n = grid * grid * ppc
    return {"workload": desc, "particles": n, "grid": [grid, grid], "dt": 0.05,
            "l2": "inputs larger than L2 (particle state %.1f GB in the mixed form)" % (n * 20e-9)}


def make_ctx(grid, st, precision, dt):
    from cpic_gb300 import _lib
    ctx = _lib.Context(grid, grid, st["L"], st["L"], dt, 1.0, (0.0, 0.0, 0.0), precision=precision,
                       track_ids=False, tile=TILE["tile"], halo=TILE["halo"])
    return ctx


def run_ours(args):
    from cpic_gb300 import _lib, build
    build.build()
    ws, rank = dist()
    grid, ppc, v0, vth, amp, desc = WORKLOADS[args.workload]
    dt = 0.05
    st = make_state(grid, ppc, v0, vth, amp, seed=2024 + rank)
    n = st["n"]
    ng = grid * grid
    form = args.precision
    prec = _lib.MIXED if form == "mixed" else _lib.FP64

    # ---- device-resident throughput (value)
    ctx = make_ctx(grid, st, prec, dt)
    ctx.add_species(st["q"], st["m"], st["x"], st["y"], st["ux"], st["uy"])
    ctx.pre_step()
    # the sampler goes live before the warm-up steps, which then keep the
    # GPU busy up to the timed region
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    if args.warmup:
        ctx.run(args.warmup)
    barrier()
    clocks.mark_start()
    t = ctx.time_steps(args.steps)
    clocks.mark_end()
    clk = clocks.stop()
    ms_total = max_over_ranks(t["ms_total"])
    barrier()
    we_series = None
    ms_step = ms_total / args.steps
    value = ws * n * args.steps / (ms_total / 1e3)
    push_ms = t["ms_plasma"] / args.steps
    field_ms = t["ms_field"] / args.steps
    tile = ctx.tile_info()
    ctx.close()

    pk, pk_kind = peaks()
    peak = float(pk.get("hbm_gbs", 6800.0))
    algo_bytes = B_P[form] * n
    achieved = algo_bytes / (push_ms / 1e3) / 1e9
    tpp = profile_traffic(form)
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_kind": pk_kind,
            "kernel": "k_push (fused gather/push/re-bin/deposit)",
            "algorithmic_bytes_per_launch": algo_bytes,
            "traffic": (tpp * n if tpp else None)}

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 particle/field math, i32 cells, i64 fixed-point charge, f64 diagnostics"
           if form == "mixed" else "f64",
           "data": DATA, "config": bench_config(grid, ppc, desc),
           "precision": "mixed" if form == "mixed" else "fp64 plain",
           "tile": tile, "parallelism": "replicas" if ws > 1 else "single GPU",
           "ms_breakdown": {"particle_kernel": push_ms, "field_stage": field_ms},
           "roofline": roof, "clocks": clk,
           # per step, either form, one species: k_rows_fwd, k_cols, k_rows_inv,
           # k_E_*, k_spill, k_push, k_tile_order (and the memsets of rho
           # and of the spill count, not counted)
           "gpu_launches": args.steps * KERNELS_PER_STEP}

    # ---- FP64 plain form on the same workload and the same window of the
    # run (after the same warm-up): the speed-up against it
    if form == "mixed" and not args.no_fp64:
        ctx64 = make_ctx(grid, st, _lib.FP64, dt)
        ctx64.add_species(st["q"], st["m"], st["x"], st["y"], st["ux"], st["uy"])
        ctx64.pre_step()
        if args.warmup:
            ctx64.run(args.warmup)
        k64 = max(2, args.steps // 4)
        t64 = ctx64.time_steps(k64)
        ctx64.close()
        ms64 = t64["ms_total"] / k64
        v64 = ws * n / (ms64 / 1e3)
        out["fp64_plain"] = {"value": v64, "ms_per_step": ms64, "steps": k64,
                             "particle_kernel_ms": t64["ms_plasma"] / k64}
        # its roofline: the FP64 pipe.  Every FP64 instruction (add, multiply,
        # conversion, compare) takes one issue slot of that pipe; the peak is
        # the measured FP64 FMA rate (instructions/s = GFLOP/s / 2), the
        # instructions per particle come from the ncu counts in profiles/
        ipp = profile_value("fp64_pipe_inst_per_particle")
        fpp = profile_value("fp64_flops_per_particle")
        try:
            g64, _ = _lib.fp64_peak()
        except Exception:
            g64 = None
        if ipp and g64:
            kt = out["fp64_plain"]["particle_kernel_ms"] / 1e3
            ach = ipp * n / kt / 1e9
            peak = g64 / 2.0
            out["fp64_plain"]["roofline"] = {
                "bound": "fp64 pipe", "achieved": round(ach, 1), "peak": round(peak, 1),
                "unit": "G FP64 instructions/s", "frac": round(ach / peak, 4),
                "peak_kind": "measured (cpic_fp64_peak: %.1f GFLOP/s of FP64 FMA chains)" % g64,
                "kernel": "k_push<F64>", "fp64_inst_per_particle": ipp,
                "flops_per_particle": fpp,
                "gflops": round(fpp * n / kt / 1e9, 1) if fpp else None}
        out["speedup_vs_fp64"] = value / v64
        # accuracy of the mixed form against the FP64 form, same initial
        # state, through the whole run: field-energy error in the linear
        # phase, growth rate and total-energy drift
        if args.accuracy_steps > 0:
            acc = accuracy_pair(grid, st, dt, args.accuracy_steps, args.linear_steps)
            out["we_rel_err_vs_fp64"] = {"steps": acc["linear_steps"],
                                         "max": acc["we_rel_err_max_linear"]}
            out["accuracy_vs_fp64"] = {k: acc[k] for k in (
                "steps", "linear_steps", "we_rel_err_max_linear", "we_rel_err_max_all",
                "growth_window_steps", "growth_rate_fp64", "growth_rate_mixed", "growth_rate_rel_err",
                "energy_drift_fp64", "energy_drift_mixed")}

    # ---- end to end through the C ABI with host buffers
    if not args.no_e2e:
        e2e_steps = max(args.steps, args.e2e_steps)
        from cpic_gb300 import _lib as L
        host, outx = pinned_state(st, n)
        barrier()
        t0 = time.perf_counter()
        ctx = make_ctx(grid, st, prec, dt)
        ctx.add_species(st["q"], st["m"], host["x"], host["y"], host["ux"], host["uy"])
        ctx.pre_step()
        ta = time.perf_counter()
        for k in range(e2e_steps):
            ctx.run(1)
            we = ctx.field_energy()
        tb = time.perf_counter()
        ctx.lib.cpic_get_particles(ctx.h, 0, *[L._dp(a) for a in outx])
        t1 = time.perf_counter()
        ctx.close()
        el = max_over_ranks(t1 - t0)
        out["e2e"] = {"value": ws * n * e2e_steps / el, "unit": UNIT, "steps": e2e_steps,
                      "seconds": el,
                      "seconds_breakdown": {"create_upload_prestep": ta - t0, "steps": tb - ta,
                                            "download": t1 - tb},
                      "h2d_bytes_per_step": 4 * 8 * n / e2e_steps,
                      "d2h_bytes_per_step": 4 * 8 * n / e2e_steps + 5 * 8,
                      "host_memory": "pinned" if host["x"].base is not None else "pageable",
                      "path": "cpic_create/cpic_add_species/cpic_pre_step, per step cpic_run(1) + "
                              "cpic_field_energy read-back, cpic_get_particles"}

    # ---- the FP64 plain form on the two-species Bz workload (GPU and oracle)
    if rank == 0 and ws == 1 and not args.no_c2:
        out["two_species_fp64"] = c2_record(args.warmup)

    # ---- CPU baseline: the oracle on a bounded sample of the workload
    if rank == 0 and ws == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(grid, ppc, v0, vth, amp, dt, n)
    return out


def pinned_state(st, n):
    """The initial state and the download buffers in page-locked host
    memory (filled before the timed region)."""
    try:
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError
        def buf():
            return torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
        host = {}
        for k in ("x", "y", "ux", "uy"):
            host[k] = buf()
            np.copyto(host[k], st[k])
        return host, [buf() for _ in range(4)]
    except Exception:
        return {k: st[k] for k in ("x", "y", "ux", "uy")}, [np.empty(n) for _ in range(4)]


C2 = dict(grid=512, ppc=16, vth_e=0.05, mass_ratio=100.0, vth_i=0.005, Bz=0.5, dt=0.05, steps=500,
          desc="two species 512x512, 16 electrons + 16 ions per cell (8,388,608 particles), "
               "Maxwellian vth 0.05 / 0.005, mass ratio 100, Bz 0.5, dt 0.05, 500 steps, FP64 plain")


def _c2_species(init):
    """Electron and ion arrays of the two-species workload from an init
    function with the (seed, species, n, Lx, Ly, vth) signature."""
    L = 2 * math.pi
    n = C2["grid"] ** 2 * C2["ppc"]
    qe = -L * L / n
    e = init(4321, 0, n, L, L, C2["vth_e"])
    i = init(4321, 1, n, L, L, C2["vth_i"])
    return [(qe, -qe, e), (-qe, -qe * C2["mass_ratio"], i)], n


def c2_record(warmup):
    """The FP64 plain form on the two-species Bz workload over its 500 steps
    (CUDA events, after the iteration-0 half kick and `warmup` steps), beside
    the oracle on one host core (full size, 1 warm-up + 2 timed steps)."""
    from cpic_gb300 import _lib
    L = 2 * math.pi
    sp, n = _c2_species(_lib.init_maxwellian)
    ctx = _lib.Context(C2["grid"], C2["grid"], L, L, C2["dt"], 1.0, (0.0, 0.0, C2["Bz"]),
                       precision=_lib.FP64, track_ids=False)
    for q, m, (x, y, ux, uy) in sp:
        ctx.add_species(q, m, x, y, ux, uy)
    del sp
    ctx.pre_step()
    ctx.run(1 + warmup)
    t = ctx.time_steps(C2["steps"])
    ctx.close()
    total = 2 * n
    v = total * C2["steps"] / (t["ms_total"] / 1e3)
    # the oracle on the same state, one core
    from oracle.oracle import Oracle, init_maxwellian
    sp, _ = _c2_species(init_maxwellian)
    o = Oracle(C2["grid"], C2["grid"], L, L, C2["dt"], 1.0, (0.0, 0.0, C2["Bz"]))
    for q, m, (x, y, ux, uy) in sp:
        o.add_species(q, m, x, y, ux, uy)
    del sp
    o.pre_step()
    o.step()
    o.step()
    t0 = time.perf_counter()
    o.step()
    o.step()
    cs = (time.perf_counter() - t0) / 2
    o.close()
    cpu = total / cs
    return {"workload": C2["desc"], "particles": total, "value": v, "unit": UNIT,
            "ms_per_step": t["ms_total"] / C2["steps"], "steps": C2["steps"],
            "particle_kernel_ms": t["ms_plasma"] / C2["steps"],
            "cpu_baseline": {"value": cpu, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": "oracle on the full workload (8,388,608 particles), 1 warm-up "
                                       "+ 2 timed steps after the half kick: %.3f s per step" % cs},
            "speedup_vs_cpu_core": v / cpu}


def _oracle_replica(grid, n, v0, vth, amp, dt, seed, warmup, steps, barrier=None, out=None):
    """The oracle (FP64 C restatement of the reference's step) on the full
    grid with n particles of the workload's seeded two-stream state: pre-step,
    `warmup` untimed steps, then `steps` steps timed one by one on the host
    clock, as the reference's own per-iteration timer does (sim.c:447-466).
    Builds its input with the oracle's own init (no product library).  With
    a barrier, every replica starts its timed steps together.  Returns (n,
    t_start, t_end, per-step seconds, field-solve seconds per step)."""
    from oracle.oracle import Oracle, init_two_stream
    L = 2 * math.pi
    x, y, ux, uy = init_two_stream(seed, 0, n, L, L, v0, vth, amp)
    q = -L * L / n
    o = Oracle(grid, grid, L, L, dt, 1.0, (0.0, 0.0, 0.0))
    o.add_species(q, -q, x, y, ux, uy)
    del x, y, ux, uy
    o.pre_step()
    for _ in range(warmup):
        o.step()
    if barrier is not None:
        barrier.wait()
    t_start = time.perf_counter()
    per_step, field = [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        o.stage_field_E()
        t1 = time.perf_counter()
        o.stage_plasma_E()
        if o.stage_plasma_r():
            raise RuntimeError("oracle step failed (velocity above umax)")
        o.stage_field_rho()
        o.iter = o.iter + 1
        t2 = time.perf_counter()
        per_step.append(t2 - t0)
        field.append(t1 - t0)
    t_end = time.perf_counter()
    o.close()
    res = (n, t_start, t_end, per_step, statistics.mean(field))
    if out is not None:
        out.put(res)
    return res


# The reference is built here against an FFTW stand-in (the oracle's FFT).
# On a side that is not a power of two its mixed-radix path takes about
# 1.5 s per field solve at 1920x1920 (0.5 s at 2048x2048 by radix 2), several
# times what FFTW needs, which would overstate the reference's step: the
# reference arm skips such grids.
NO_REF_GRID = ("grid side not a power of two: the FFTW stand-in the reference is built against "
               "here transforms such sides several times slower than FFTW (about 1.5 s per "
               "field solve at 1920x1920), which would overstate the reference's step")


def pow2_grid(grid):
    return grid > 0 and grid & (grid - 1) == 0


def cpu_baseline(grid, ppc, v0, vth, amp, dt, n_full):
    """One core: the oracle on the full grid with 1/16 of the workload's
    particles (all of them below 1024^2), 1 warm-up and 3 timed steps; the
    per-particle cost and the field-solve cost are scaled to the workload."""
    frac = 1.0 / 16 if grid >= 1024 else 1.0
    n = max(1024, int(n_full * frac))
    n, t0, t1, per_step, tf = _oracle_replica(grid, n, v0, vth, amp, dt, 99, 1, 3)
    tp = (statistics.mean(per_step) - tf) / n
    per_full = n_full * tp + tf
    return {"value": n_full / per_full, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "oracle (FP64 C restatement of the reference step) on the full %dx%d grid "
                      "with %d particles (1/%d of the workload), 1 warm-up + 3 timed steps; particle "
                      "cost %.1f ns/particle-step and field solve %.3f s/step scaled to %d particles"
                      % (grid, grid, n, round(1 / frac), tp * 1e9, tf, n_full)}


def run_reference(args):
    """The reference on the host cores, on the workload: one process per core,
    each on the full grid with 1/cores of the workload's particles (so that
    together they step the workload's particle count), W warm-up steps, then
    K steps timed together (a barrier starts them).  value = particles
    stepped by all processes x K / wall time of that window.  The processes
    run the reference's own code, built from its sources (oracle/build_ref.py,
    with the portable intrinsics on the Arm host) when it is built here,
    else its C restatement, the oracle.  Loads no product library and uses no
    GPU."""
    ws, rank = dist()
    if rank != 0:
        return None
    grid, ppc, v0, vth, amp, desc = WORKLOADS[args.workload]
    if not pow2_grid(grid):
        return {"impl": "reference", "unavailable": NO_REF_GRID}
    from oracle import ref_run
    cores = os.cpu_count() or 1
    n_full = grid * grid * ppc
    n = max(1024, n_full // cores)
    L = 2 * math.pi
    if ref_run.harness() is not None:
        res = ref_run.time_two_stream(cores, grid, n, v0, vth, amp, 0.05, L, args.warmup, args.steps)
        res = [(r[0], r[1], r[2], list(r[3]), None) for r in res]
        kind = "reference"
        what = ("the reference's own step (src/*.c as shipped, built from its sources against "
                "single-rank MPI/FFTW/libconfig stand-ins, serial), driven by oracle/ref_harness.c")
    else:
        from oracle import oracle
        oracle.build()
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        barrier, q = ctx.Barrier(cores), ctx.Queue()
        procs = [ctx.Process(target=_oracle_replica,
                             args=(grid, n, v0, vth, amp, 0.05, 99 + i, args.warmup, args.steps, barrier, q))
                 for i in range(cores)]
        for p in procs:
            p.start()
        res = [q.get() for _ in procs]
        for p in procs:
            p.join()
            if p.exitcode != 0:
                raise RuntimeError("oracle replica failed (exit code %s)" % p.exitcode)
        kind = "port"
        what = ("the oracle (FP64 C restatement of the reference step, single threaded; the "
                "reference itself is not built on this host)")
    window = max(r[2] for r in res) - min(r[1] for r in res)
    total = sum(r[0] for r in res)
    v = total * args.steps / window
    ms_step = window / args.steps * 1e3
    mean_step = statistics.mean(statistics.mean(r[3]) for r in res)
    sample = ("%d concurrent processes of %s, one per host core, each the full %dx%d grid with "
              "%d of the workload's particles (%d in all), %d warm-up + %d timed steps; mean step "
              "%.3f s per process" % (cores, what, grid, grid, n, total, args.warmup, args.steps,
                                      mean_step))
    return {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": DATA, "config": bench_config(grid, ppc, desc),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def _growth_rate(t, we):
    """Least-squares slope of ln(W_E) / 2 (field amplitude growth rate)."""
    t = np.asarray(t)
    y = np.log(np.asarray(we))
    A = np.vstack([t, np.ones_like(t)]).T
    slope = np.linalg.lstsq(A, y, rcond=None)[0][0]
    return 0.5 * slope


def study_phases(args):
    """Step time through the whole run of the workload (mixed form), in
    blocks of 50 CUDA-event-timed steps, each followed by 10 steps with a
    field-energy read-back after every step (host-timed), with the layout
    statistics and the spread of tile counts (largest and 99th percentile
    over the mean) at the end of each block.  The two-stream run goes
    through a linear phase, then bunches (tile counts up to 3.6x the mean,
    tile overflows, layout rebuilds) and mixes in velocity."""
    from cpic_gb300 import _lib, build
    build.build()
    grid, ppc, v0, vth, amp, desc = WORKLOADS[args.workload]
    st = make_state(grid, ppc, v0, vth, amp)
    ctx = make_ctx(grid, st, _lib.MIXED, 0.05)
    ctx.add_species(st["q"], st["m"], st["x"], st["y"], st["ux"], st["uy"])
    del st
    ctx.pre_step()
    T = ctx.tile_info()["tile_x"]
    rows, done, blk = [], 0, 50
    while done < args.study_steps:
        t = ctx.time_steps(blk)
        done += blk
        stats = ctx.layout_stats()
        tc = ctx.cell_counts().astype(np.int64).reshape(grid // T, T, grid // T, T).sum(axis=(1, 3))
        t1 = time.perf_counter()
        for _ in range(10):
            ctx.run(1)
            ctx.field_energy()
        ms_sync = (time.perf_counter() - t1) * 100
        done += 10
        rows.append({"step": done, "ms_step": t["ms_total"] / blk, "ms_push": t["ms_plasma"] / blk,
                     "ms_field": t["ms_field"] / blk, "ms_step_synced": ms_sync, "stats": stats,
                     "tile_max_over_mean": float(tc.max() / tc.mean()),
                     "tile_p99_over_mean": float(np.quantile(tc, 0.99) / tc.mean()),
                     "field_energy": ctx.field_energy()})
    # the same state re-laid out with 100 % slack (not 200 %): whether the
    # late steps' cost comes from the store's spread (slack grown to 200 %)
    before = ctx.layout_stats()
    ctx.compact(100)
    t = ctx.time_steps(blk)
    rows.append({"step": done + blk, "after_compact_to_100pct": True, "slack_before": before["slack_pct"],
                 "ms_step": t["ms_total"] / blk, "ms_push": t["ms_plasma"] / blk,
                 "ms_field": t["ms_field"] / blk, "stats": ctx.layout_stats()})
    # the same particles uploaded again into a fresh context: the upload sort
    # orders every tile's particles by direction of motion, in place of the
    # order the in-place re-bin has accumulated (arrival order); the steps
    # after it show what that order costs (timing only: the new context's
    # iteration 0 is a half kick)
    n = ctx.counts[0]
    L = 2 * math.pi
    H = ctx.tile_info()["halo"]
    x, y, ux, uy = ctx.particles(0)
    ctx.close()
    q = -L * L / n
    # same tile, halo (so the same resident blocks per SM) and slack
    ctx = _lib.Context(grid, grid, L, L, 0.05, 1.0, (0.0, 0.0, 0.0), precision=_lib.MIXED,
                       track_ids=False, tile=T, halo=H)
    ctx.add_species(q, -q, x, y, ux, uy)
    del x, y, ux, uy
    ctx.pre_step()
    ctx.compact(200)
    ctx.run(1)
    t = ctx.time_steps(blk)
    rows.append({"step": done + 2 * blk + 1, "after_reupload": True, "ms_step": t["ms_total"] / blk,
                 "ms_push": t["ms_plasma"] / blk, "ms_field": t["ms_field"] / blk,
                 "stats": ctx.layout_stats()})
    ctx.close()
    return {"study": "phases", "workload": desc, "tile": T, "rows": rows}


def accuracy_pair(grid, st, dt, steps, lin):
    """Mixed form against the FP64 form from the same initial state, `steps`
    steps with the FP64 diagnostics after each: field-energy error through
    the linear phase (steps 1..lin) and overall, growth rate of the field
    amplitude fitted in the exponential window of the FP64 run, and the
    drift of the total energy (field + kinetic) over the run."""
    from cpic_gb300 import _lib
    ctx = {}
    for name, prec in (("fp64", _lib.FP64), ("mixed", _lib.MIXED)):
        c = make_ctx(grid, st, prec, dt)
        c.add_species(st["q"], st["m"], st["x"], st["y"], st["ux"], st["uy"])
        c.pre_step()
        ctx[name] = c
    series = {k: {"we": [], "tot": []} for k in ctx}
    d0 = {name: c.diag() for name, c in ctx.items()}
    for k in range(steps):
        for name, c in ctx.items():
            c.step()
            d = c.diag()
            series[name]["we"].append(d["WE"])
            series[name]["tot"].append(d["WE"] + d["KE"])
    for c in ctx.values():
        c.close()
    lin = min(lin, steps)
    we64 = np.array(series["fp64"]["we"])
    wem = np.array(series["mixed"]["we"])
    rel = np.abs(wem - we64) / we64
    t = dt * np.arange(1, steps + 1)
    # exponential phase of the FP64 run: from W_E rising above 10x its
    # noise level (median over the first lin steps) to 30% of its peak
    base = float(np.median(we64[:lin]))
    above = np.nonzero(we64 > 10.0 * base)[0]
    top = np.nonzero(we64 >= 0.3 * we64.max())[0]
    i0 = int(above[0]) if len(above) else lin // 6
    i1 = int(top[0]) if len(top) else lin
    if i1 - i0 < 20:
        i0, i1 = max(1, lin // 6), lin
    win = slice(i0, i1)
    res = {"steps": steps, "linear_steps": lin,
           "we_rel_err_max_linear": float(rel[:lin].max()),
           "we_rel_err_max_all": float(rel.max()),
           "growth_window_steps": [win.start + 1, win.stop]}
    for name in ("fp64", "mixed"):
        we = np.array(series[name]["we"])
        tot = np.array(series[name]["tot"])
        e0 = d0[name]["WE"] + d0[name]["KE"]
        res["growth_rate_" + name] = float(_growth_rate(t[win], we[win]))
        res["energy_drift_" + name] = float((tot[-1] - e0) / e0)
        res["we_final_" + name] = float(we[-1])
        res["we_max_" + name] = float(we.max())
    res["growth_rate_rel_err"] = abs(res["growth_rate_mixed"] - res["growth_rate_fp64"]) / abs(
        res["growth_rate_fp64"])
    every = max(1, steps // 50)
    res["we_samples"] = {"step": list(range(1, steps + 1, every)),
                         "fp64": [float(v) for v in we64[::every]],
                         "mixed": [float(v) for v in wem[::every]]}
    return res


def study_accuracy(args):
    """Mixed form against the FP64 form on the same workload from the same
    initial state (accuracy_pair), no timing."""
    from cpic_gb300 import build
    build.build()
    grid, ppc, v0, vth, amp, desc = WORKLOADS[args.workload]
    st = make_state(grid, ppc, v0, vth, amp)
    res = accuracy_pair(grid, st, 0.05, args.study_steps, args.linear_steps)
    res.update({"study": "accuracy", "workload": desc})
    return res


def ensemble_members(nruns, seed=2024):
    """Seeded ensemble: grid side from {32, 64, 128, 256}, 8-128 particles
    per cell, beam speed in [0.1, 0.4], perturbation amplitude in
    [0.001, 0.05]; cold two-stream beams, dt 0.05, L = 2 pi."""
    rng = np.random.default_rng(seed)
    grid = rng.choice([32, 64, 128, 256], nruns)
    ppc = rng.integers(8, 129, nruns)
    v0 = rng.uniform(0.1, 0.4, nruns)
    amp = rng.uniform(0.001, 0.05, nruns)
    return [dict(grid=int(g), ppc=int(c), v0=float(v), amp=float(a), seed=i + 1)
            for i, (g, c, v, a) in enumerate(zip(grid, ppc, v0, amp))]


def _member_ctx(m, precision, tile, ppt=0):
    from cpic_gb300 import _lib
    L = 2 * math.pi
    n = m["grid"] * m["grid"] * m["ppc"]
    x, y, ux, uy = _lib.init_two_stream(m["seed"], 0, n, L, L, m["v0"], 0.0, m["amp"])
    q = -L * L / n
    c = _lib.Context(m["grid"], m["grid"], L, L, 0.05, 1.0, (0.0, 0.0, 0.0), precision=precision,
                     track_ids=False, tile=tile, ppt=ppt)
    c.add_species(q, -q, x, y, ux, uy)
    c.pre_step()
    return c, n


def _oracle_member_step_s(m, timed=2):
    """Seconds per step of the oracle on one ensemble member (same state
    as _member_ctx), after its pre-step and one warm-up step."""
    from oracle.oracle import Oracle, init_two_stream
    L = 2 * math.pi
    n = m["grid"] * m["grid"] * m["ppc"]
    x, y, ux, uy = init_two_stream(m["seed"], 0, n, L, L, m["v0"], 0.0, m["amp"])
    q = -L * L / n
    o = Oracle(m["grid"], m["grid"], L, L, 0.05, 1.0, (0.0, 0.0, 0.0))
    o.add_species(q, -q, x, y, ux, uy)
    o.pre_step()
    o.step()
    t0 = time.perf_counter()
    for _ in range(timed):
        o.step()
    dt = (time.perf_counter() - t0) / timed
    o.close()
    return dt


def ensemble_cpu_baseline(members, steps, threads):
    """The ensemble on the host cores, one oracle process per run as the
    reference would run it (one run per job): every member's cost per step
    is timed on a bounded sample (2 steps after its pre-step and one
    warm-up step, `threads` members at a time), scaled to `steps` steps,
    and the runs are packed onto `threads` cores longest first."""
    import heapq
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(threads) as pool:
        per_step = pool.map(_oracle_member_step_s, members, chunksize=1)
    sample_wall = time.perf_counter() - t0
    work = sorted((steps * s for s in per_step), reverse=True)
    cores = [0.0] * threads
    for w in work:
        heapq.heapreplace(cores, cores[0] + w)
    makespan = max(cores)
    return {"value": len(members) / makespan, "unit": "runs/s", "cores": threads, "kind": "port",
            "seconds_estimated": makespan, "cpu_seconds": sum(work),
            "sample": "oracle (FP64 C restatement of the reference step), one process per run on "
                      "%d host cores: each run's step cost timed over 2 steps after its pre-step "
                      "and one warm-up step (%.1f s wall for all %d runs), scaled to %d steps, runs "
                      "packed onto the cores longest first" % (threads, sample_wall, len(members),
                                                                steps)}


def study_ensemble(args):
    """Batched ensemble: every run of the ensemble stepped by one CUDA graph
    (after autotuning the tile per (grid, particles per cell)), against the
    same runs stepped one after another; per-run field-energy error of the
    mixed form against the FP64 form over the first 300 steps."""
    from cpic_gb300 import _lib, build
    import torch
    build.build()
    L = 2 * math.pi
    members = ensemble_members(args.ensemble_runs)
    steps = args.ensemble_steps
    t0 = time.perf_counter()
    tiles = {}
    for m in members:
        key = (m["grid"], int(round(math.log2(m["ppc"]))))
        if key not in tiles:
            n = m["grid"] * m["grid"] * m["ppc"]
            tiles[key] = _lib.autotune_layout(m["grid"], m["grid"], L, L, 0.05, n, m["v0"], 0.0)[:2]
        m["tile"], m["ppt"] = tiles[key]
    t_tune = time.perf_counter() - t0
    res = {"study": "ensemble", "runs": len(members), "steps": steps, "precision": "mixed",
           "particles_total": int(sum(m["grid"] ** 2 * m["ppc"] for m in members)),
           "autotune_seconds": t_tune,
           "autotuned_layouts": {"%dx%d ppc~2^%d" % (k[0], k[0], k[1]): {"tile": v[0], "ppt": v[1]}
                                 for k, v in sorted(tiles.items())}}
    pstep = res["particles_total"] * steps
    # one graph for all runs
    runs = [_member_ctx(m, _lib.MIXED, m["tile"], m["ppt"])[0] for m in members]
    ens = _lib.Ensemble(runs)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ms_graph, caps = ens.run(steps)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    res.update({"graph_wall_s": wall, "graph_ms_device": ms_graph, "graph_captures": caps,
                "runs_per_s": len(members) / wall, "particle_steps_per_s": pstep / wall})
    ens.close()
    for c in runs:
        c.close()
    del runs
    # the same runs one after another, no graph
    t_seq = 0.0
    for m in members:
        c, n = _member_ctx(m, _lib.MIXED, m["tile"], m["ppt"])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c.run(steps)
        torch.cuda.synchronize()
        t_seq += time.perf_counter() - t0
        c.close()
    res.update({"sequential_wall_s": t_seq, "sequential_runs_per_s": len(members) / t_seq,
                "graph_speedup": t_seq / wall})
    # per-run error against the FP64 form
    if not args.no_fp64:
        lin = min(300, steps)
        errs = []
        for m in members:
            cm, _ = _member_ctx(m, _lib.MIXED, m["tile"], m["ppt"])
            cf, _ = _member_ctx(m, _lib.FP64, 0)
            worst = 0.0
            for k in range(0, lin, 20):
                cm.run(20)
                cf.run(20)
                a, b = cm.field_energy(), cf.field_energy()
                worst = max(worst, abs(a - b) / b)
            errs.append(worst)
            cm.close()
            cf.close()
        errs = np.array(errs)
        res.update({"we_rel_err_vs_fp64": {"steps": lin, "median": float(np.median(errs)),
                                           "p90": float(np.quantile(errs, 0.9)),
                                           "max": float(errs.max()),
                                           "runs_below_1e-5": int(np.sum(errs <= 1e-5))}})
    # the same runs on the host cores, one oracle process per run
    if not args.no_cpu:
        res["cpu_baseline"] = ensemble_cpu_baseline(members, steps, os.cpu_count() or 1)
        res["runs_per_s_over_cpu"] = res["runs_per_s"] / res["cpu_baseline"]["value"]
    return res


def study_adjoint(args):
    """Adjoint of the field energy after 200 steps (128x128, 64 electrons
    per cell, v0 0.2, amplitude 0.01, checkpoint every 20): cost against the
    forward run, FP64 and FP32, and the gradients with respect to v0 and the
    amplitude against FP64 central finite differences (eps 1e-6)."""
    from cpic_gb300 import _lib, build
    build.build()
    L = 2 * math.pi
    grid, ppc, steps, K = 128, 64, 200, 20
    n = grid * grid * ppc
    q = -L * L / n
    xt, y, _, _ = _lib.init_two_stream(11, 0, n, L, L, 1.0, 0.0, 0.0)
    sign = np.where(np.arange(n) < n // 2, 1.0, -1.0)
    sx = np.sin(2 * math.pi * xt / L)
    zeros = np.zeros(n)

    def state(v0, amp):
        return np.mod(xt + amp * sx, L), y, sign * v0, zeros

    res = {"study": "adjoint", "grid": grid, "particles": n, "steps": steps, "checkpoint_every": K}
    fd = {}
    for name, prec in (("fp64", _lib.FP64), ("fp32", _lib.MIXED)):
        adj = _lib.Adjoint(grid, grid, L, L, 0.05, 1.0, q, -q, n, steps, K, precision=prec)
        adj.forward(*state(0.2, 0.01))
        adj.backward()
        loss = adj.forward(*state(0.2, 0.01))
        g = adj.backward()
        tf, tb = adj.times()
        dv0 = float(np.sum(sign * g[2]))
        damp = float(np.sum(sx * g[0]))
        r = {"loss": loss, "dL_dv0": dv0, "dL_damp": damp, "ms_forward": tf, "ms_backward": tb,
             "backward_over_forward": tb / tf}
        if prec == _lib.FP64:
            res["fd_fp64"] = {}
            for eps in (1e-6, 1e-8):
                fv = (adj.forward(*state(0.2 + eps, 0.01)) - adj.forward(*state(0.2 - eps, 0.01))) / (2 * eps)
                fa = (adj.forward(*state(0.2, 0.01 + eps)) - adj.forward(*state(0.2, 0.01 - eps))) / (2 * eps)
                fd[eps] = (fv, fa)
                res["fd_fp64"]["eps=%g" % eps] = {"dL_dv0": fv, "dL_damp": fa}
        r["rel_err_vs_fd"] = {"eps=%g" % eps: {"v0": abs(dv0 - f[0]) / abs(f[0]),
                                               "amp": abs(damp - f[1]) / abs(f[1])}
                              for eps, f in fd.items()}
        res[name] = r
        adj.close()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="two_stream_2048", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--accuracy-steps", type=int, default=1000,
                    help="steps of the mixed-vs-FP64 comparison in the default line (the "
                    "workload's run length; 0 skips it)")
    ap.add_argument("--linear-steps", type=int, default=300,
                    help="steps of the linear phase for the field-energy error bound")
    ap.add_argument("--study", default="", choices=["", "accuracy", "ensemble", "adjoint", "phases"],
                    help="accuracy: long mixed-vs-FP64 run (growth rate, energy drift), no timing; "
                    "ensemble: batched independent runs in one CUDA graph; adjoint: gradient "
                    "cost and finite-difference check; phases: step time through the whole "
                    "run (--study-steps), with layout statistics")
    ap.add_argument("--ensemble-runs", type=int, default=256)
    ap.add_argument("--ensemble-steps", type=int, default=400)
    ap.add_argument("--study-steps", type=int, default=1000)
    ap.add_argument("--e2e-steps", type=int, default=1000,
                    help="steps of the end-to-end run: the workload's run length (1000 steps)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-c2", action="store_true", help="skip the two-species FP64 record")
    ap.add_argument("--tile", type=int, default=0, help="tile size in cells (0: library default)")
    ap.add_argument("--halo", type=int, default=0, help="deposit halo in cells (0: library default)")
    args = ap.parse_args()
    TILE["tile"], TILE["halo"] = args.tile, args.halo
    args.warmup = max(args.warmup, 0)
    ws, rank = dist()
    if ws > 1:
        import torch
        import torch.distributed as td
        td.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        if torch.cuda.is_available():
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if args.study == "accuracy":
        out = study_accuracy(args) if rank == 0 else None
    elif args.study == "ensemble":
        out = study_ensemble(args) if rank == 0 else None
    elif args.study == "adjoint":
        out = study_adjoint(args) if rank == 0 else None
    elif args.study == "phases":
        out = study_phases(args) if rank == 0 else None
    else:
        out = run_reference(args) if args.impl == "reference" else run_ours(args)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if ws > 1:
        import torch.distributed as td
        td.destroy_process_group()


if __name__ == "__main__":
    main()
