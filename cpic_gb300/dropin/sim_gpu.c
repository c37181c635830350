/* sim_gpu.c -- drop-in replacement for cpic's src/sim.c that runs the time
 * step on the GPU library (libcpic_gb300, include/cpic_gpu.h).
 *
 * It is compiled inside the host cpic tree, against that tree's own headers
 * (def.h, sim.h, plist.h, ...), in place of src/sim.c; every other host
 * file (config, species, field/plasma allocation, particle init methods,
 * plist, perf, output) is kept and linked unchanged.  Exports exactly the
 * three entry points of src/sim.h:9-15:
 *
 *   sim_t *sim_init(config_t *conf, int quiet);   src/sim.c:238
 *   int    sim_step(sim_t *sim);                  src/sim.c:481
 *   int    sim_run(sim_t *sim);                   src/sim.c:621
 *
 * with the reference's semantics: sim_init reads the same mandatory keys
 * (sim.c:37-80), prepares the same derived sizes (sim.c:82-203), builds the
 * host species, fields and plasma with the host's own initialisers and
 * init methods, then does the pre-step (sim.c:208-236) on the GPU and
 * leaves iter = 0.  sim_step returns -1 once iter >= cycles, advances iter
 * and t, keeps the "stats" sampling line and the stop_SEM criterion
 * (sim.c:431-479).  Errors return NULL / -1 instead of aborting.
 *
 * Host views.  Callers (test/constant-speed.c, test/cyclotron.c, the field
 * writer) read the ppacks and sim->field directly.  After a step the
 * particles (r, u, and E interpolated at the pre-push position, as
 * stage_plasma_E leaves it) are written back into the chunks' plists and
 * rho, phi, E into the field views every `gpu.host_sync` steps (default 1;
 * 0 = only when fields are written and at the end of sim_run).  The
 * environment variable CPIC_GPU_HOST_SYNC overrides the config.
 *
 * Optional config group (absent in the reference's .conf files):
 *   gpu = { precision = "fp64" | "mixed"; host_sync = 1;
 *           tile = [tx, ty]; halo = h; };
 * and, per species, an initial state the reference's init methods
 * (particle.c:170-175) cannot express, applied after them:
 *   gpu_init = { method = "two stream"; v0 = 0.2; vth = 0.01; amp = 0.01;
 *                seed = 1; };                     (cpic_init_two_stream)
 *   gpu_init = { method = "maxwellian"; vth = 0.05; drift = [0.0, 0.0];
 *                seed = 1; };                     (cpic_init_maxwellian)
 *
 * Limits: one MPI process (the GPU library owns the whole domain), the
 * "MFT" solver only, 2D, in-plane velocities (u_z = 0) and B along z.
 */
#define _GNU_SOURCE
#include <assert.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/resource.h>

#include <libconfig.h>
#include <mpi.h>

#include "sim.h"
#include "def.h"
#include "config.h"
#include "field.h"
#include "output.h"
#include "perf.h"
#include "plasma.h"
#include "plist.h"
#include "solver.h"
#include "specie.h"

#include "cpic_gpu.h"

/* Per-sim state of the GPU side.  sim_t has no spare field, so it hangs off
 * the sim's solver: sim->solver is a real solver_t (method "MFT", no FFTW
 * plans: the GPU library owns the solve) whose `data` member, the slot the
 * reference keeps for a solver's own state (solver.h:41), points here. */
struct gpu_sim
{
	cpic_ctx_t *ctx;
	int host_sync;          /* sync period in steps, 0 = on demand only */
	int64_t *n;             /* particles per species */
	int64_t **pid;          /* per species: reference particle index by GPU id */
	double *buf;            /* 4 * max(n) doubles: x y ux uy */
	double *ebuf;           /* 2 * sum(n) doubles: E at the particles */
	double *fbuf;           /* 2 * nx * (ny + 1) doubles */
	int views_due;          /* host views are refreshed by this step's stages */
	int e_pending;          /* ebuf holds E gathered before this step's push */
	int err;                /* a stage failed: later stages and sim_step fail too */
};

#define GPU(sim) ((sim)->solver ? (struct gpu_sim *) (sim)->solver->data : NULL)

static void
gpu_err(const char *what, int rc)
{
	fprintf(stderr, "sim_gpu: %s failed with status %d\n", what, rc);
}

/* ---------------------------------------------------------------------
 * Configuration (same mandatory keys as sim_read_config, sim.c:37-80)
 * --------------------------------------------------------------------- */

static int
read_config(sim_t *s)
{
	config_t *conf = s->conf;

#define MUST(call, key) \
	if((call) != CONFIG_TRUE) { fprintf(stderr, "sim_gpu: missing parameter \"%s\"\n", key); return 1; }

	MUST(config_lookup_i64(conf, "simulation.dimensions", &s->dim), "simulation.dimensions");
	MUST(config_lookup_i64(conf, "simulation.cycles", &s->cycles), "simulation.cycles");
	MUST(config_lookup_float(conf, "simulation.time_step", &s->dt), "simulation.time_step");
	MUST(config_lookup_int(conf, "simulation.random_seed", (int *) &s->seed), "simulation.random_seed");
	MUST(config_lookup_float(conf, "constants.light_speed", &s->C), "constants.light_speed");
	MUST(config_lookup_float(conf, "constants.vacuum_permittivity", &s->e0),
			"constants.vacuum_permittivity");
	MUST(config_lookup_i64(conf, "simulation.sampling_period.energy", &s->period_energy),
			"simulation.sampling_period.energy");
	MUST(config_lookup_i64(conf, "simulation.sampling_period.field", &s->period_field),
			"simulation.sampling_period.field");
	MUST(config_lookup_i64(conf, "simulation.sampling_period.particle", &s->period_particle),
			"simulation.sampling_period.particle");
	MUST(config_lookup_float(conf, "simulation.stop_SEM", &s->stop_SEM), "simulation.stop_SEM");
	MUST(config_lookup_int(conf, "simulation.realtime_plot", &s->mode), "simulation.realtime_plot");
	MUST(config_lookup_string(conf, "simulation.solver", &s->solver_method), "simulation.solver");
	MUST(config_lookup_i64(conf, "simulation.enable_fftw_threads", &s->fftw_threads),
			"simulation.enable_fftw_threads");
	MUST(config_lookup_i64(conf, "simulation.plasma_chunks", &s->plasma_chunks),
			"simulation.plasma_chunks");
	MUST(config_lookup_i64(conf, "simulation.pblock_nmax", &s->pblock_nmax),
			"simulation.pblock_nmax");
#undef MUST

	config_lookup_array_float(conf, "simulation.space_length", s->L, s->dim);
	for(i64 d = s->dim; d < MAX_DIM; d++) s->L[d] = 0;
	config_lookup_array_float(conf, "field.magnetic", s->B, MAX_DIM);
	config_lookup_array_int(conf, "grid.points", s->ntpoints, s->dim);
	s->nspecies = config_setting_length(config_lookup(conf, "species"));
	return 0;
}

/* Derived sizes, as sim_prepare (sim.c:82-203) computes them. */
static int
prepare(sim_t *s, int quiet)
{
	MPI_Comm_rank(MPI_COMM_WORLD, &s->rank);
	MPI_Comm_size(MPI_COMM_WORLD, &s->nprocs);
	if(s->nprocs != 1)
	{
		fprintf(stderr, "sim_gpu: one process per simulation (got %d)\n", s->nprocs);
		return 1;
	}
	if(s->dim != 2)
	{
		fprintf(stderr, "sim_gpu: only 2 dimensions are supported\n");
		return 1;
	}
	if(strcmp(s->solver_method, "MFT") != 0)
	{
		fprintf(stderr, "sim_gpu: solver \"%s\" not available, only \"MFT\"\n", s->solver_method);
		return 1;
	}
	if(s->plasma_chunks <= 0 || (s->ntpoints[X] % s->plasma_chunks) != 0)
	{
		fprintf(stderr, "sim_gpu: grid points in X %ld not divisible by plasma_chunks %ld\n",
				(long) s->ntpoints[X], (long) s->plasma_chunks);
		return 1;
	}
	if(s->B[X] != 0.0 || s->B[Y] != 0.0)
	{
		fprintf(stderr, "sim_gpu: only a magnetic field along z is supported\n");
		return 1;
	}

	s->iter = -2;
	s->running = 1;
	s->sampling = s->stop_SEM > 0.0;
	if(quiet) s->mode = SIM_MODE_NORMAL;
	s->run = 1;
	srand(s->seed + (unsigned int) s->rank);
	s->ghostpoints = 1;
	s->nneigh_chunks = 3;
	s->desired_mxcsr = 0;

	for(int d = s->dim; d < MAX_DIM; d++)
	{
		s->ntpoints[d] = 1;
		s->dx[d] = 0.0;
		s->chunksize[d] = 1;
		s->blocksize[d] = 1;
	}
	for(int d = 0; d < s->dim; d++)
		s->dx[d] = s->L[d] / s->ntpoints[d];

	s->blocksize[X] = s->ntpoints[X];
	s->blocksize[Y] = s->ntpoints[Y];
	s->blocksize[Z] = s->ntpoints[Z];
	s->ghostsize[X] = s->blocksize[X];
	s->ghostsize[Y] = s->blocksize[Y] + s->ghostpoints;
	s->ghostsize[Z] = s->blocksize[Z];
	s->chunksize[X] = s->blocksize[X] / s->plasma_chunks;
	s->chunksize[Y] = s->blocksize[Y];
	s->chunksize[Z] = s->blocksize[Z];
	s->proc_table = calloc((size_t) s->nprocs, sizeof(s->proc_table[0]));

	for(int d = 0; d < MAX_DIM; d++)
		s->umax[d] = s->chunksize[d] * s->dx[d] / s->dt;
	s->t = 0.0;
	return 0;
}

/* ---------------------------------------------------------------------
 * Host views: ppacks <-> flat arrays, fields
 * --------------------------------------------------------------------- */

/* Copies the particles of species `is` out of every chunk's plist. */
static int64_t
collect_species(sim_t *sim, int is, double *x, double *y, double *ux, double *uy, int64_t *pid,
		int64_t cap)
{
	int64_t k = 0;
	for(i64 ic = 0; ic < sim->plasma.nchunks; ic++)
	{
		plist_t *l = &sim->plasma.chunks[ic].species[is].list;
		for(pblock_t *b = l->b; b; b = b->next)
		{
			for(i64 j = 0; j < b->n; j++)
			{
				ppack_t *p = &b->p[j / MAX_VEC];
				int iv = (int) (j % MAX_VEC);
				if(k >= cap) return -1;
				if(p->u[Z][iv] != 0.0) return -2;
				x[k] = p->r[X][iv];
				y[k] = p->r[Y][iv];
				ux[k] = p->u[X][iv];
				uy[k] = p->u[Y][iv];
				pid[k] = p->i[iv];
				k++;
			}
		}
	}
	return k;
}

/* Rewrites the plists of species `is` from the flat arrays (GPU id order):
 * each particle goes to the chunk whose [x0, x1) holds it; garbage lanes of
 * the last pack get the chunk's x0 and zero velocity and field, as the
 * reference leaves them (comm_plasma.c:659-692). */
static void
scatter_species(sim_t *sim, int is, int64_t n, const double *x, const double *y,
		const double *ux, const double *uy, const double *ex, const double *ey,
		const int64_t *pid)
{
	i64 nc = sim->plasma.nchunks;
	double wchunk = sim->chunksize[X] * sim->dx[X];
	for(i64 ic = 0; ic < nc; ic++)
	{
		pchunk_t *chunk = &sim->plasma.chunks[ic];
		plist_t *l = &chunk->species[is].list;
		double x0 = chunk->x0[X][0];
		int64_t cnt = 0;
		for(int64_t k = 0; k < n; k++)
		{
			i64 c = (i64) (x[k] / wchunk);
			if(c >= nc) c = nc - 1;
			if(c == ic) cnt++;
		}
		plist_clear(l);
		for(int64_t left = cnt; left > 0; )
		{
			int64_t g = left < l->nmax ? left : l->nmax;
			plist_grow(l, g);
			left -= g;
		}
		pblock_t *b = l->b;
		i64 j = 0;
		for(int64_t k = 0; k < n; k++)
		{
			i64 c = (i64) (x[k] / wchunk);
			if(c >= nc) c = nc - 1;
			if(c != ic) continue;
			while(j >= b->n) { b = b->next; j = 0; }
			ppack_t *p = &b->p[j / MAX_VEC];
			int iv = (int) (j % MAX_VEC);
			p->magic[iv] = MAGIC_PARTICLE;
			p->i[iv] = pid[k];
			p->r[X][iv] = x[k]; p->r[Y][iv] = y[k]; p->r[Z][iv] = 0.0;
			p->u[X][iv] = ux[k]; p->u[Y][iv] = uy[k]; p->u[Z][iv] = 0.0;
			p->E[X][iv] = ex ? ex[k] : 0.0; p->E[Y][iv] = ey ? ey[k] : 0.0; p->E[Z][iv] = 0.0;
			for(int d = 0; d < MAX_DIM; d++) p->B[d][iv] = sim->B[d];
			j++;
		}
		/* garbage lanes of the last, partial pack of every block */
		for(b = l->b; b; b = b->next)
		{
			if(b->n % MAX_VEC == 0) continue;
			ppack_t *p = &b->p[b->n / MAX_VEC];
			for(int iv = (int) (b->n % MAX_VEC); iv < MAX_VEC; iv++)
			{
				p->magic[iv] = MAGIC_GARBAGE;
				p->i[iv] = -1;
				for(int d = 0; d < MAX_DIM; d++)
				{
					p->r[d][iv] = d == X ? x0 : 0.0;
					p->u[d][iv] = 0.0;
					p->E[d][iv] = 0.0;
					p->B[d][iv] = 0.0;
				}
			}
		}
	}
}

/* Copies an ny x nx row-major array into a mat view, plus `ghost` extra
 * rows that repeat rows 0.. periodically. */
static void
fill_view(mat_t *m, const double *v, i64 nx, i64 ny, i64 ghost)
{
	for(i64 iy = 0; iy < ny + ghost; iy++)
		for(i64 ix = 0; ix < nx; ix++)
			MAT_XY(m, ix, iy) = v[(iy % ny) * nx + ix];
}

static int
sync_fields(sim_t *sim)
{
	struct gpu_sim *g = GPU(sim);
	field_t *f = &sim->field;
	i64 nx = sim->ntpoints[X], ny = sim->ntpoints[Y];
	int rc;
	if((rc = cpic_get_rho(g->ctx, g->fbuf))) { gpu_err("cpic_get_rho", rc); return -1; }
	fill_view(f->rho, g->fbuf, nx, ny, 0);
	if((rc = cpic_get_phi(g->ctx, g->fbuf))) { gpu_err("cpic_get_phi", rc); return -1; }
	fill_view(f->phi, g->fbuf, nx, ny, 0);
	/* E comes with its south ghost row: (ny + 1) x nx per component */
	i64 ne = nx * (ny + E_NG_SOUTH);
	if((rc = cpic_get_E(g->ctx, g->fbuf, g->fbuf + ne))) { gpu_err("cpic_get_E", rc); return -1; }
	fill_view(f->E[X], g->fbuf, nx, ny + E_NG_SOUTH, 0);
	fill_view(f->E[Y], g->fbuf + ne, nx, ny + E_NG_SOUTH, 0);
	return 0;
}

/* Particle write-back.  ebuf (may be NULL): per species, the E gathered
 * before the push (ex then ey, species after species). */
static int
sync_particles(sim_t *sim, const double *ebuf)
{
	struct gpu_sim *g = GPU(sim);
	for(int is = 0; is < (int) sim->nspecies; is++)
	{
		int64_t n = g->n[is];
		double *x = g->buf, *y = x + n, *ux = y + n, *uy = ux + n;
		int rc;
		if((rc = cpic_get_particles(g->ctx, is, x, y, ux, uy)))
		{
			gpu_err("cpic_get_particles", rc);
			return -1;
		}
		scatter_species(sim, is, n, x, y, ux, uy, ebuf, ebuf ? ebuf + n : NULL, g->pid[is]);
		if(ebuf) ebuf += 2 * n;
	}
	return 0;
}

/* ---------------------------------------------------------------------
 * GPU context
 * --------------------------------------------------------------------- */

static double
conf_float(config_setting_t *g, const char *name, double dflt)
{
	double v;
	int i;
	if(config_setting_lookup_float(g, name, &v) == CONFIG_TRUE) return v;
	if(config_setting_lookup_int(g, name, &i) == CONFIG_TRUE) return i;
	return dflt;
}

/* The species' gpu_init group, if any, replaces the state the host's init
 * method produced (same particle count; ids are kept). */
static int
apply_gpu_init(sim_t *sim, int is, int64_t n, double *x, double *y, double *ux, double *uy)
{
	config_setting_t *gi = config_setting_get_member(sim->species[is].conf, "gpu_init");
	const char *method = NULL;
	int seed = (int) sim->seed;
	if(!gi) return 0;
	if(config_setting_lookup_string(gi, "method", &method) != CONFIG_TRUE)
	{
		fprintf(stderr, "sim_gpu: species %d: gpu_init without a method\n", is);
		return 1;
	}
	config_setting_lookup_int(gi, "seed", &seed);
	if(!strcmp(method, "two stream"))
		cpic_init_two_stream((uint64_t) seed, is, n, sim->L[X], sim->L[Y],
				conf_float(gi, "v0", 0.0), conf_float(gi, "vth", 0.0),
				conf_float(gi, "amp", 0.0), x, y, ux, uy);
	else if(!strcmp(method, "maxwellian"))
	{
		double drift[2] = {0.0, 0.0};
		config_setting_t *d = config_setting_get_member(gi, "drift");
		if(d && config_setting_length(d) == 2)
		{
			drift[0] = config_setting_get_float_elem(d, 0);
			drift[1] = config_setting_get_float_elem(d, 1);
		}
		cpic_init_maxwellian((uint64_t) seed, is, n, sim->L[X], sim->L[Y],
				conf_float(gi, "vth", 0.0), drift[0], drift[1], x, y, ux, uy);
	}
	else
	{
		fprintf(stderr, "sim_gpu: species %d: unknown gpu_init method \"%s\"\n", is, method);
		return 1;
	}
	return 0;
}

static int
gpu_setup(sim_t *sim)
{
	struct gpu_sim *g = calloc(1, sizeof(*g));
	const char *prec = "fp64", *env;
	config_setting_t *gs;
	cpic_params_t p;
	int rc, sync = 1;
	int64_t nmax = 1;

	if(!g) return 1;
	sim->solver = calloc(1, sizeof(solver_t));
	if(!sim->solver) return 1;
	sim->solver->method = METHOD_MFT;
	sim->solver->dim = sim->dim;
	sim->solver->nx = sim->ntpoints[X];
	sim->solver->ny = sim->ntpoints[Y];
	sim->solver->data = g;

	memset(&p, 0, sizeof(p));
	p.nx = sim->ntpoints[X];
	p.ny = sim->ntpoints[Y];
	p.Lx = sim->L[X];
	p.Ly = sim->L[Y];
	p.dt = sim->dt;
	p.e0 = sim->e0;
	for(int d = 0; d < 3; d++) p.B[d] = sim->B[d];
	p.plasma_chunks = sim->plasma_chunks;
	p.cycles = sim->cycles;
	p.track_ids = 1;
	if((gs = config_lookup(sim->conf, "gpu")))
	{
		config_setting_t *t;
		int v;
		config_setting_lookup_string(gs, "precision", &prec);
		if(config_setting_lookup_int(gs, "host_sync", &v) == CONFIG_TRUE) sync = v;
		if(config_setting_lookup_int(gs, "halo", &v) == CONFIG_TRUE) p.halo = v;
		if((t = config_setting_get_member(gs, "tile")) && config_setting_length(t) == 2)
		{
			p.tile_x = config_setting_get_int_elem(t, 0);
			p.tile_y = config_setting_get_int_elem(t, 1);
		}
	}
	if((env = getenv("CPIC_GPU_HOST_SYNC"))) sync = atoi(env);
	g->host_sync = sync < 0 ? 0 : sync;
	if(!strcmp(prec, "fp64")) p.precision = CPIC_FP64;
	else if(!strcmp(prec, "mixed")) p.precision = CPIC_MIXED;
	else
	{
		fprintf(stderr, "sim_gpu: unknown gpu.precision \"%s\"\n", prec);
		return 1;
	}

	if((rc = cpic_create(&p, &g->ctx))) { gpu_err("cpic_create", rc); return 1; }

	g->n = calloc((size_t) sim->nspecies, sizeof(int64_t));
	g->pid = calloc((size_t) sim->nspecies, sizeof(int64_t *));
	for(int is = 0; is < (int) sim->nspecies; is++)
	{
		int64_t n = 0;
		for(i64 ic = 0; ic < sim->plasma.nchunks; ic++)
			n += plist_get_n(&sim->plasma.chunks[ic].species[is].list);
		g->n[is] = n;
		if(n > nmax) nmax = n;
	}
	int64_t ntot = 0;
	for(int is = 0; is < (int) sim->nspecies; is++) ntot += g->n[is];
	g->buf = malloc(4 * (size_t) nmax * sizeof(double));
	g->ebuf = malloc(2 * (size_t) (ntot ? ntot : 1) * sizeof(double));
	g->fbuf = malloc(2 * (size_t) p.nx * (size_t) (p.ny + 1) * sizeof(double));
	if(!g->buf || !g->ebuf || !g->fbuf) return 1;

	for(int is = 0; is < (int) sim->nspecies; is++)
	{
		int64_t n = g->n[is];
		double *x = g->buf, *y = x + n, *ux = y + n, *uy = ux + n;
		g->pid[is] = malloc((size_t) (n ? n : 1) * sizeof(int64_t));
		int64_t got = collect_species(sim, is, x, y, ux, uy, g->pid[is], n);
		if(got == -2)
		{
			fprintf(stderr, "sim_gpu: species %d has u_z != 0 (in-plane motion only)\n", is);
			return 1;
		}
		if(got != n) return 1;
		if(apply_gpu_init(sim, is, n, x, y, ux, uy)) return 1;
		rc = cpic_add_species(g->ctx, sim->species[is].q, sim->species[is].m, n, x, y, ux, uy);
		if(rc < 0) { gpu_err("cpic_add_species", rc); return 1; }
	}
	return 0;
}

/* ---------------------------------------------------------------------
 * sim.h entry points
 * --------------------------------------------------------------------- */

sim_t *
sim_init(config_t *conf, int quiet)
{
	sim_t *s = calloc(1, sizeof(sim_t));
	int rc;

	if(!s) return NULL;
	s->conf = conf;
	if(read_config(s) || prepare(s, quiet))
		return NULL;

	if(species_init(s))
		return NULL;
	s->output = calloc(1, sizeof(*s->output));
	if(!s->output || output_init(s, s->output))
		return NULL;
	if(field_init(s, &s->field))
		return NULL;
	if(plasma_init(s, &s->plasma))
		return NULL;

	s->iter++;                              /* -1: the pre-step */
	s->t = s->iter * s->dt;
	if(gpu_setup(s))
		return NULL;
	if((rc = cpic_pre_step(GPU(s)->ctx)))
	{
		gpu_err("cpic_pre_step", rc);
		return NULL;
	}
	if(sync_fields(s) || sync_particles(s, NULL))
		return NULL;

	s->iter++;
	s->t = s->iter * s->dt;
	assert(s->iter == 0);
	return s;
}

/* The "stats" line and stop_SEM criterion of the reference's sampling
 * mode (sim.c:431-479). */
static int
sampling_done(sim_t *sim)
{
	double t = perf_measure(&sim->timers[TIMER_ITERATION]);
	double ts = perf_measure(&sim->timers[TIMER_SOLVER]);
	double mean, std, sem, ms, ss, es, rsem;
	struct rusage u;

	perf_stats(&sim->timers[TIMER_ITERATION], &mean, &std, &sem);
	perf_record(&sim->timers[TIMER_ITERATION], t);
	perf_stats(&sim->timers[TIMER_SOLVER], &ms, &ss, &es);
	perf_record(&sim->timers[TIMER_SOLVER], ts);
	rsem = mean != 0.0 ? sem / mean : sem;
	getrusage(RUSAGE_SELF, &u);
	printf("stats iter=%ld last=%e mean=%e std=%e sem=%e rsem=%e mem=%ld solver=%e\n",
			(long) sim->iter, t, mean, std, sem, rsem, (long) u.ru_maxrss, ms);
	if(sim->iter < 30) return 0;
	return 1.96 * sem < sim->stop_SEM * mean;
}

/* ---------------------------------------------------------------------
 * Stage entry points, with the reference's prototypes (field.h:9-12,
 * particle.h:20-26, mover.h:4, comm.h:38).  The GPU fuses the gather, the
 * push with the periodic re-bin and the deposit into one kernel, so:
 *
 *   stage_field_E    rho -> phi -> E on the GPU (field.c:451); refreshes the
 *                    host field views when they are due or when output is
 *                    enabled (sim_step then calls the reference's
 *                    output_fields, as sim.c:507 does);
 *   stage_plasma_E   E at the particles (particle.c:233): on the GPU this is
 *                    part of the next stage; when host views are due it
 *                    gathers E at the pre-push positions into the ppacks'
 *                    E, as the reference leaves it;
 *   stage_plasma_r   the fused gather + Boris push + wrap + re-bin + charge
 *                    deposit (mover.c:332 with comm_plasma, and the deposit
 *                    of field.c:269);
 *   stage_field_rho  the deposit is already done: refreshes the host views
 *                    of rho and of the particles when they are due;
 *   comm_plasma, particle_comm_initial
 *                    the re-bin is part of stage_plasma_r and of the
 *                    pre-step; nothing is left to exchange (one process).
 *
 * Host views are due on steps that are multiples of gpu.host_sync.  The
 * reference aborts on a failing stage; the void stages here print the
 * status and set a sticky error that makes every later stage a no-op and
 * sim_step return -1.  A caller that runs the stages itself, as sim_step
 * does, advances sim->iter after stage_field_rho.
 * --------------------------------------------------------------------- */

static int
views_due(sim_t *sim, struct gpu_sim *g)
{
	return g->host_sync > 0 && (sim->iter % g->host_sync) == 0;
}

int
stage_field_E(sim_t *sim)
{
	struct gpu_sim *g = GPU(sim);
	int rc;
	if(!g || g->err) return -1;
	g->views_due = views_due(sim, g);
	if((rc = cpic_stage_field_E(g->ctx)))
	{
		gpu_err("cpic_stage_field_E", rc);
		g->err = rc;
		return -1;
	}
	if((g->views_due || sim->output->enabled) && sync_fields(sim))
	{
		g->err = CPIC_ECUDA;
		return -1;
	}
	return 0;
}

void
stage_plasma_E(sim_t *sim)
{
	struct gpu_sim *g = GPU(sim);
	int rc;
	if(!g || g->err) return;
	g->e_pending = 0;
	if(!g->views_due) return;
	double *e = g->ebuf;
	for(int is = 0; is < (int) sim->nspecies; is++)
	{
		if((rc = cpic_gather_E(g->ctx, is, e, e + g->n[is])))
		{
			gpu_err("cpic_gather_E", rc);
			g->err = rc;
			return;
		}
		e += 2 * g->n[is];
	}
	g->e_pending = 1;
}

void
stage_plasma_r(sim_t *sim)
{
	struct gpu_sim *g = GPU(sim);
	int rc;
	if(!g || g->err) return;
	if((rc = cpic_stage_plasma(g->ctx)))
	{
		gpu_err("cpic_stage_plasma", rc);
		g->err = rc;
	}
}

void
stage_field_rho(sim_t *sim)
{
	struct gpu_sim *g = GPU(sim);
	if(!g || g->err) return;
	if(g->views_due && (sync_fields(sim) || sync_particles(sim, g->e_pending ? g->ebuf : NULL)))
		g->err = CPIC_ECUDA;
	g->views_due = 0;
	g->e_pending = 0;
}

int
comm_plasma(sim_t *sim, int global_exchange)
{
	(void) global_exchange;
	struct gpu_sim *g = GPU(sim);
	return (!g || g->err) ? -1 : 0;
}

int
particle_comm_initial(sim_t *sim)
{
	return comm_plasma(sim, 1);
}

int
sim_step(sim_t *sim)
{
	struct gpu_sim *g = GPU(sim);
	int rc;

	if(sim->iter < 0 || !g || g->err) return -1;
	if(sim->iter >= sim->cycles) return -1;

	perf_reset(&sim->timers[TIMER_ITERATION]);
	perf_start(&sim->timers[TIMER_ITERATION]);

	if(views_due(sim, g) || sim->output->enabled)
	{
		/* the reference's stage sequence (sim.c:509-565), with the host
		 * views refreshed between the stages */
		if(stage_field_E(sim))
			return -1;
		if(output_fields(sim))
		{
			fprintf(stderr, "sim_gpu: output_fields failed\n");
			return -1;
		}
		stage_plasma_E(sim);
		stage_plasma_r(sim);
		stage_field_rho(sim);
		if(g->err)
			return -1;
	}
	else if((rc = cpic_step(g->ctx)))
	{
		/* no host views this step: the whole step in one call */
		gpu_err("cpic_step", rc);
		g->err = rc;
		return -1;
	}

	perf_stop(&sim->timers[TIMER_ITERATION]);
	if(sim->sampling && sampling_done(sim))
	{
		printf("sampling complete\n");
		sim->running = 0;
	}
	sim->iter += 1;
	sim->t = sim->iter * sim->dt;
	return 0;
}

int
sim_run(sim_t *sim)
{
	if(!sim || sim->iter != 0) return -1;
	perf_start(&sim->timers[TIMER_TOTAL]);
	if(sim->rank == 0)
		printf("Simulation runs now\n");
	while(sim->running && sim->iter < sim->cycles)
	{
		if(sim_step(sim))
		{
			fprintf(stderr, "sim_step failed\n");
			return -1;
		}
	}
	sim->running = 0;
	perf_stop(&sim->timers[TIMER_TOTAL]);
	/* final host view */
	if(sync_fields(sim) || sync_particles(sim, NULL))
		return -1;
	return 0;
}
