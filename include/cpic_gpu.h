/*
 * cpic_gpu.h -- C ABI of the GB300 implementation of cpic's 2D
 * electrostatic PIC time step.
 *
 * One context holds one simulation resident in GPU memory: the particle
 * store (structure of arrays, sorted by tile), the fields and the Poisson
 * solver.  The entry points mirror the reference's simulation-loop and
 * stage functions; each comment names the reference function it replaces
 * (file:line inside the rodarima/cpic tree).  Arguments are plain host
 * pointers and sizes; every call is synchronous with respect to the host
 * unless stated otherwise.
 *
 * Error convention: 0 on success, a negative CPIC_E* code on failure.  The
 * reference aborts on these conditions (src/mover.c:97-137, src/utils.c);
 * this library never aborts and never traps on the device: kernels record
 * errors in a status word that the next host-side check turns into a code.
 */
#ifndef CPIC_GPU_H
#define CPIC_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CPIC_API __attribute__((visibility("default")))

enum cpic_precision {
	/* FP64 positions and velocities, reference arithmetic order, no FMA
	 * contraction: one-step positions are bit-exact with the reference. */
	CPIC_FP64 = 0,
	/* int32 cell index + FP32 in-cell offset, FP32 velocity and E;
	 * charge reduction, k=0 removal and diagnostics in FP64/int64. */
	CPIC_MIXED = 1,
};

enum cpic_status {
	CPIC_OK = 0,
	CPIC_EINVAL = -1,     /* bad argument or unsupported configuration */
	CPIC_ENOMEM = -2,     /* device or host allocation failed */
	CPIC_ECUDA = -3,      /* CUDA runtime error */
	CPIC_EUMAX = -4,      /* |u| > umax: the reference aborts (mover.c:97) */
	CPIC_ENAN = -5,       /* non-finite particle state */
	CPIC_ECAPACITY = -6,  /* particle store could not hold a tile */
	CPIC_EDONE = -7,      /* iter >= cycles (sim_step returns -1, sim.c:486) */
	CPIC_ENODEV = -8,     /* no CUDA device */
	CPIC_ESTATE = -9,     /* call out of order (e.g. step before pre_step) */
	CPIC_ETIMEOUT = -10,  /* a bounded device-side wait expired */
};

/* Simulation parameters; the .conf key each field comes from is named.
 * Defaults for zero fields: plasma_chunks 1, tile and halo chosen by the
 * library, 2 particles per thread.  No reference counterpart for the last
 * four (the reference's blocks are MPI ranks and plasma chunks). */
typedef struct cpic_params {
	int64_t nx, ny;          /* grid.points: any size, 4 ... 16384 */
	double Lx, Ly;           /* simulation.space_length */
	double dt;               /* simulation.time_step */
	double e0;               /* constants.vacuum_permittivity */
	double B[3];             /* field.magnetic (only B[Z] may be non-zero) */
	int64_t plasma_chunks;   /* simulation.plasma_chunks (sets umax) */
	int64_t cycles;          /* simulation.cycles */
	int32_t precision;       /* enum cpic_precision */
	int32_t tile_x, tile_y;  /* cells per tile, equal powers of two dividing
	                          * nx and ny; 0 = auto */
	int32_t halo;            /* deposit halo in cells; 0 = auto */
	int32_t track_ids;       /* keep a particle id per particle (MIXED) */
	int32_t particles_per_thread; /* fused kernel instance: 1, 2 or 4; 0 = chosen
	                               * at cpic_add_species: 1 while every species
	                               * has < 4096 particles per tile, else 2 */
	int32_t reserved[6];
} cpic_params_t;

typedef struct cpic_ctx cpic_ctx_t;

/* --- lifecycle ----------------------------------------------------- */

/* Allocates the fields, the solver tables and the (empty) particle store
 * on the current CUDA device.  Replaces sim_init's set-up half
 * (src/sim.c:238-303: sim_prepare sim.c:87, field_init field.c:20,
 * plasma_init plasma.c:293, solver_init solver.c:551). */
CPIC_API int cpic_create(const cpic_params_t *p, cpic_ctx_t **out);

/* Frees everything.  Replaces sim_end/solver_end (sim.c:322, solver.c:628). */
CPIC_API void cpic_destroy(cpic_ctx_t *ctx);

/* Adds one species with n particles (host FP64 arrays, positions inside
 * [0,Lx) x [0,Ly) up to one periodic image in Y).  Replaces specie_init +
 * pset_init + particles_init (specie.c:14, plasma.c:20, particle.c:177).
 * Returns the species index (>= 0) or an error code. */
CPIC_API int cpic_add_species(cpic_ctx_t *ctx, double q, double m, int64_t n,
		const double *x, const double *y, const double *ux, const double *uy);

/* Global re-bin, initial charge deposit and first field solve, leaving
 * iter = 0.  Replaces sim_pre_step (sim.c:208-236). */
CPIC_API int cpic_pre_step(cpic_ctx_t *ctx);

/* --- time stepping -------------------------------------------------- */

/* One full step: field solve + E, then the fused gather / Boris push /
 * re-bin / deposit kernel.  Iteration 0 is the backward half kick
 * (mover.c:204-213).  Returns CPIC_EDONE when iter >= cycles.
 * Replaces sim_step (sim.c:481-581). */
CPIC_API int cpic_step(cpic_ctx_t *ctx);

/* nsteps calls of cpic_step, launched without host synchronisation in
 * between (one status check at the end).  Replaces sim_run (sim.c:621). */
CPIC_API int cpic_run(cpic_ctx_t *ctx, int64_t nsteps);

/* rho -> phi -> E.  Replaces stage_field_E (field.c:450-501): solve_xy /
 * MFT_solve (solver.c:598, 465), the phi ghost exchange
 * (comm_field.c:140-201) and field_E_compute (field.c:358-416). */
CPIC_API int cpic_stage_field_E(cpic_ctx_t *ctx);

/* Gather E to every particle, Boris push, periodic wrap, re-bin and
 * charge deposit, fused.  Replaces stage_plasma_E (particle.c:232),
 * stage_plasma_r (mover.c:331) with comm_plasma (comm_plasma.c:1123) and
 * stage_field_rho (field.c:268) with the ghost fold
 * (comm_field.c:52-136).  Advances iter by one. */
CPIC_API int cpic_stage_plasma(cpic_ctx_t *ctx);

/* --- host views ------------------------------------------------------ */

CPIC_API int64_t cpic_iter(const cpic_ctx_t *ctx);
CPIC_API int cpic_nspecies(const cpic_ctx_t *ctx);
CPIC_API int64_t cpic_species_count(const cpic_ctx_t *ctx, int species);

/* Particle state of one species as FP64, ordered by particle id (the
 * index at cpic_add_species) when ids are tracked, else in store order.
 * Any pointer may be NULL.  The host view the reference keeps in its
 * ppacks (def.h:88-98). */
CPIC_API int cpic_get_particles(cpic_ctx_t *ctx, int species, double *x,
		double *y, double *ux, double *uy);

/* Overwrites positions/velocities of one species (ids order, FP64).
 * Used to inject the same state into the oracle and the GPU. */
CPIC_API int cpic_set_particles(cpic_ctx_t *ctx, int species,
		const double *x, const double *y, const double *ux, const double *uy);

/* E at every particle for the current fields and positions (ids order),
 * as interpolate_f2p_E computes it (interpolate.c:349-404). */
CPIC_API int cpic_gather_E(cpic_ctx_t *ctx, int species, double *ex, double *ey);

/* Fields, FP64, row-major (row = y).  rho and phi: ny x nx (the views
 * without FFT padding or ghosts, field.c:83-118); E: (ny+1) x nx with the
 * south ghost row (field.c:123-132). */
CPIC_API int cpic_get_rho(cpic_ctx_t *ctx, double *rho);
CPIC_API int cpic_get_phi(cpic_ctx_t *ctx, double *phi);
CPIC_API int cpic_get_E(cpic_ctx_t *ctx, double *ex, double *ey);
CPIC_API int cpic_set_E(cpic_ctx_t *ctx, const double *ex, const double *ey);
CPIC_API int cpic_set_rho(cpic_ctx_t *ctx, const double *rho);

/* Particles per cell, ny x nx (cell = floor of the position over dx). */
CPIC_API int cpic_cell_counts(cpic_ctx_t *ctx, int64_t *counts);

/* FP64 diagnostics on the device, out[5] = {field energy
 * 0.5 e0 sum|E|^2 dx dy, kinetic energy 0.5 sum m|u|^2, total charge
 * sum(rho) dx dy, momentum x, momentum y}.  The reference's energy
 * diagnostic is compiled out (sim.c:332-405). */
CPIC_API int cpic_diag(cpic_ctx_t *ctx, double *out);

/* Field energy only (out[0]) and total charge (out[1]), O(grid): the
 * per-step scalar a driver reads back.  Same definitions as cpic_diag. */
CPIC_API int cpic_field_energy(cpic_ctx_t *ctx, double *out);

/* Device status word (bit field, 0 = healthy) without clearing it. */
CPIC_API uint32_t cpic_status_bits(cpic_ctx_t *ctx);

/* No counterpart in the reference (it aborts instead of waiting).  Self-test
 * of the device-side bounded wait that every kernel of this library uses
 * on its shared-memory pipeline: one warp waits, with at most `polls` probes
 * (each may suspend the thread for the hardware's time limit; at most the
 * kernels' own limit of 2^20), on an mbarrier phase that never completes.  It is armed for
 * the bytes of a copy that is never issued, so nothing is in flight.
 * Returns CPIC_ETIMEOUT when the wait expired and the kernel returned, as it
 * must; the device stays usable afterwards. */
CPIC_API int cpic_selftest_wait(uint32_t polls);

/* --- measurement ------------------------------------------------------ */

/* Runs nsteps steps timed with CUDA events on the context's stream.
 * ms_total: whole interval; ms_plasma: summed duration of the fused
 * particle kernel; ms_field: summed duration of the field stage.  No
 * host synchronisation inside the interval. */
CPIC_API int cpic_time_steps(cpic_ctx_t *ctx, int64_t nsteps, double *ms_total,
		double *ms_plasma, double *ms_field);

/* No counterpart in the reference.  FP64 arithmetic peak of the current
 * device, the denominator of the FP64 form's roofline: every thread of
 * enough resident blocks runs independent chains of `iters` dependent FP64
 * FMAs (2 FLOPs each), timed with CUDA events after one shorter warm-up
 * launch.  gflops: measured GFLOP/s; ms (may be NULL): the timed launch.
 * Changes no device setting. */
CPIC_API int cpic_fp64_peak(int64_t iters, double *gflops, double *ms);

/* No counterpart in the reference (its particle blocks grow and shrink by
 * list).  Re-lays the particle store out with `slack_pct` percent of spare
 * capacity per tile (a counting-sort rebuild from the current state; the
 * particles and their order within a tile are kept).  Tile overflows double
 * the slack up to 200 %; a run whose particles have spread out again can
 * compact its store back.  Synchronous. */
CPIC_API int cpic_compact(cpic_ctx_t *ctx, int32_t slack_pct);

/* Tile geometry chosen for this context: out[4] = {tile_x, tile_y, halo,
 * capacity slack in percent}. */
CPIC_API int cpic_tile_info(const cpic_ctx_t *ctx, int32_t *out);

/* How the fused particle kernel stages each tile's field: *mode = 1 when
 * the mixed form copies it with one 2D tensor copy per tile (tiles of an
 * even width up to 254 cells, an even nx; tiles in the grid's last column
 * or row, whose nodes wrap, load by threads), 0 when every tile loads by
 * threads (the FP64 form reads E from global memory). */
CPIC_API int cpic_field_tile_copy(const cpic_ctx_t *ctx, int32_t *mode);

/* Health of the tile layout, out[4]: {overflow records (particles that
 * found no room in their destination tile) seen at the last host check,
 * layout rebuilds forced by overflows so far, current capacity slack in
 * percent, resident blocks per SM of the fused particle kernel at this
 * context's tile and halo (0 before the first species)}. */
CPIC_API int cpic_layout_stats(const cpic_ctx_t *ctx, int64_t *out);

/* --- solve without allocation ------------------------------------------ */

/* Largest grid side accepted by cpic_poisson_noalloc: its scratch is one
 * fixed array of about 2.1 MB held by every GPU that loads the library. */
#define CPIC_NOALLOC_MAX_N 512

/* No counterpart in the reference.  Periodic FP64 Poisson solve phi = IFFT(G
 * FFT(rho)) / (nx ny) with the reference's Green's function, for callers that
 * must not allocate device memory (a fixed memory budget or their own pool
 * owning the device, or host threads on which cudaMalloc/cudaFree and their
 * implicit synchronisation must not appear).  rho and phi are the caller's
 * device buffers, ny x nx row-major doubles; nx and ny powers of two in
 * [4, CPIC_NOALLOC_MAX_N] (larger grids are rejected with CPIC_EINVAL);
 * stream is a cudaStream_t (NULL: the default stream); asynchronous.  The
 * scratch lives in a static device array shared by all calls: the first call
 * on each device looks up its address (make that first call before any
 * stream capture), and calls that overlap on the GPU race on it. */
CPIC_API int cpic_poisson_noalloc(const double *rho, double *phi, int64_t nx, int64_t ny,
		void *stream);

/* --- ensembles of independent runs ------------------------------------ */

/* No counterpart in the reference (one run per MPI job there).  Groups
 * prepared contexts (after cpic_pre_step, on the current device; not owned
 * by the ensemble) of any grid sizes and particle counts. */
typedef struct cpic_ensemble cpic_ensemble_t;

CPIC_API int cpic_ensemble_create(cpic_ctx_t *const *runs, int32_t nruns,
		cpic_ensemble_t **out);
CPIC_API void cpic_ensemble_destroy(cpic_ensemble_t *e);

/* nsteps steps of every run.  Iteration 0 runs eagerly; then one CUDA graph
 * holding two steps of every run (each run an independent branch) is
 * captured once and relaunched, the runs' status checked every 4 steps
 * (a run whose tile layout is rebuilt causes one re-capture).  ms_graph:
 * CUDA-event time of the graph launches; captures: graphs captured so far
 * (either may be NULL). */
CPIC_API int cpic_ensemble_run(cpic_ensemble_t *e, int64_t nsteps, double *ms_graph,
		int32_t *captures);

/* Autotuner: the tile size (cells per side; it is also the counting-sort
 * bin width of the re-bin) for grid p->nx x p->ny, precision p->precision
 * and n particles, chosen by timing a seeded two-stream plasma (beam speed
 * v0, spread vth) with each candidate.  Cached per (grid, log2 particles
 * per cell, precision) for the process. */
CPIC_API int cpic_autotune_tile(const cpic_params_t *p, int64_t n, double v0, double vth,
		int32_t *tile, double *ms_per_step);

/* Autotuner over the whole layout: the tile size and the fused kernel's
 * particles per thread (its compiled instances: 1, 2 or 4 particles per
 * thread and chunk, i.e. chunks of 256, 512 or 1024 particles staged per
 * block), timed together as cpic_autotune_tile does; same cache rule. */
CPIC_API int cpic_autotune_layout(const cpic_params_t *p, int64_t n, double v0, double vth,
		int32_t *tile, int32_t *particles_per_thread, double *ms_per_step);

/* --- adjoint: gradient of the final field energy ---------------------- */

/* No counterpart in the reference.  A differentiable run of the step for one
 * species: nsteps calls of the step (iteration 0, the backward half kick,
 * included) from an initial state (x, y, ux, uy), then the loss
 * L = 1/2 e0 dx dy sum over nodes of |E|^2, with E solved from the charge of
 * the final positions.  The backward sweep gives dL/dx, dL/dy, dL/dux,
 * dL/duy of every initial particle by hand-written adjoint kernels: the
 * gather's adjoint is a deposit, the deposit's a gather of the weight
 * gradients, the Boris kick's the transposed rotation, the Poisson solve is
 * its own adjoint.  States are kept every checkpoint_every steps and
 * recomputed in between.  Precision CPIC_FP64, or CPIC_MIXED for FP32 state,
 * fields and adjoint (charge sums stay 64-bit fixed point in both). */
typedef struct cpic_adj_params {
	int64_t nx, ny;           /* powers of two */
	double Lx, Ly, dt, e0;
	double q, m;              /* the species' macro charge and mass */
	double Bz;                /* magnetic field along z */
	int64_t nsteps;           /* >= 1 */
	int64_t checkpoint_every; /* K >= 1 */
	int32_t precision;
	int32_t reserved[7];
} cpic_adj_params_t;

typedef struct cpic_adj cpic_adj_t;

CPIC_API int cpic_adj_create(const cpic_adj_params_t *p, int64_t n, cpic_adj_t **out);
CPIC_API void cpic_adj_destroy(cpic_adj_t *a);

/* Uploads the initial state (host FP64, positions in [0,Lx) x [0,Ly)),
 * runs the nsteps forward, keeping the checkpoints, and returns L. */
CPIC_API int cpic_adj_forward(cpic_adj_t *a, const double *x, const double *y,
		const double *ux, const double *uy, double *loss);

/* After cpic_adj_forward: the gradient of L with respect to the initial
 * state (host FP64 arrays of n; any may be NULL). */
CPIC_API int cpic_adj_backward(cpic_adj_t *a, double *gx, double *gy, double *gux,
		double *guy);

/* CUDA-event durations of the last forward and backward sweeps, ms. */
CPIC_API int cpic_adj_times(const cpic_adj_t *a, double *ms_forward, double *ms_backward);

/* --- seeded initial states (host only; no GPU needed) ----------------- */

/* The i-th uniform / normal draw of (seed, stream), i < n. */
CPIC_API void cpic_uniform(uint64_t seed, uint64_t stream, int64_t n, double *out);
CPIC_API void cpic_normal(uint64_t seed, uint64_t stream, int64_t n, double *out);

/* Two counter-streaming beams (+v0 for the first n/2 particles, -v0 for
 * the rest) with thermal spread vth, uniform positions displaced by
 * amp*sin(2 pi x/Lx).  New init method beside particle.c:170-175. */
CPIC_API void cpic_init_two_stream(uint64_t seed, int species, int64_t n,
		double Lx, double Ly, double v0, double vth, double amp,
		double *x, double *y, double *ux, double *uy);

/* Uniform positions, drifting 2D Maxwellian velocities.  New init
 * method beside particle.c:170-175. */
CPIC_API void cpic_init_maxwellian(uint64_t seed, int species, int64_t n,
		double Lx, double Ly, double vth, double driftx, double drifty,
		double *x, double *y, double *ux, double *uy);

#ifdef __cplusplus
}
#endif

#endif /* CPIC_GPU_H */
