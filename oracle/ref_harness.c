/*
 * ref_harness.c -- drives the reference simulation (built from the
 * reference's own sources against the shims in oracle/shims) on a given
 * particle state and dumps what the parity tests compare.
 * TEST INFRASTRUCTURE ONLY; runs as its own process because sim_init
 * enables floating-point traps (src/sim.c:102-106).
 *
 * usage: ref_harness CONF STATE_IN OUT_DIR NSTEPS [DUMP_STEPS...]
 *
 * STATE_IN holds, per species of CONF in order: int64 n, then n doubles of
 * x, y, ux, uy.  After sim_init the harness overwrites every particle of
 * the ppacks (matched by their index p->i), re-runs the pre-step stages
 * (particle_comm_initial, stage_field_rho, stage_field_E: sim.c:208-236)
 * and writes OUT_DIR/pre.bin; then it calls sim_step NSTEPS times,
 * appending the field energy of each step to OUT_DIR/energy.bin and
 * writing OUT_DIR/step<k>.bin after the steps listed.
 *
 * A dump: int64 nx, ny, nspecies; rho (ny x nx), phi (ny x nx), Ex, Ey
 * ((ny+1) x nx); per species: int64 n, then for every particle in the
 * plist order: int64 id, x, y, ux, uy, Ex, Ey.
 *
 * Timing mode (the CPU arm of the benchmark): STATE_IN of the form
 * "two_stream:SEED:V0:VTH:AMP" generates every species' state with the
 * seeded two-stream generator (seed_init.h, the product's init method)
 * instead of reading a file; NSTEPS is "WARMUP+STEPS".  After the pre-step
 * and WARMUP untimed steps the harness creates OUT_DIR/ready.<pid> and waits
 * for OUT_DIR/go (so that concurrent harnesses time the same window), then
 * times STEPS calls of sim_step and writes OUT_DIR/times.<pid>: int64
 * particles, then CLOCK_MONOTONIC seconds (double) before the first and
 * after every timed step.  No dumps in this mode.
 */
#define _GNU_SOURCE
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "seed_init.h"

#include "def.h"
#include "sim.h"
#include "field.h"
#include "particle.h"

static void
die_msg(const char *m)
{
	fprintf(stderr, "ref_harness: %s\n", m);
	exit(2);
}

static void
wr(FILE *f, const void *p, size_t n)
{
	if(fwrite(p, 1, n, f) != n) die_msg("write failed");
}

static void
dump(sim_t *sim, const char *path)
{
	FILE *f = fopen(path, "wb");
	int64_t nx = sim->blocksize[X], ny = sim->blocksize[Y], ns = sim->nspecies, ix, iy, is;
	if(!f) die_msg("cannot open dump");
	wr(f, &nx, 8); wr(f, &ny, 8); wr(f, &ns, 8);
	for(iy = 0; iy < ny; iy++)
		for(ix = 0; ix < nx; ix++)
			wr(f, &MAT_XY(sim->field.rho, ix, iy), 8);
	for(iy = 0; iy < ny; iy++)
		for(ix = 0; ix < nx; ix++)
			wr(f, &MAT_XY(sim->field.phi, ix, iy), 8);
	for(iy = 0; iy < ny + 1; iy++)
		for(ix = 0; ix < nx; ix++)
			wr(f, &MAT_XY(sim->field._E[X], ix, iy), 8);
	for(iy = 0; iy < ny + 1; iy++)
		for(ix = 0; ix < nx; ix++)
			wr(f, &MAT_XY(sim->field._E[Y], ix, iy), 8);
	for(is = 0; is < ns; is++)
	{
		int64_t n = 0, ic;
		for(ic = 0; ic < sim->plasma.nchunks; ic++)
		{
			pblock_t *b;
			for(b = sim->plasma.chunks[ic].species[is].list.b; b; b = b->next)
				n += b->n;
		}
		wr(f, &n, 8);
		for(ic = 0; ic < sim->plasma.nchunks; ic++)
		{
			pblock_t *b;
			for(b = sim->plasma.chunks[ic].species[is].list.b; b; b = b->next)
			{
				int64_t k;
				for(k = 0; k < b->n; k++)
				{
					ppack_t *p = &b->p[k / MAX_VEC];
					int iv = (int) (k % MAX_VEC);
					int64_t id = p->i[iv];
					double v[6] = {p->r[X][iv], p->r[Y][iv], p->u[X][iv], p->u[Y][iv],
						p->E[X][iv], p->E[Y][iv]};
					wr(f, &id, 8);
					wr(f, v, sizeof(v));
				}
			}
		}
	}
	fclose(f);
}

static double
field_energy(sim_t *sim)
{
	int64_t nx = sim->blocksize[X], ny = sim->blocksize[Y], ix, iy;
	double we = 0.0;
	for(iy = 0; iy < ny; iy++)
		for(ix = 0; ix < nx; ix++)
		{
			double ex = MAT_XY(sim->field.E[X], ix, iy);
			double ey = MAT_XY(sim->field.E[Y], ix, iy);
			we += ex * ex + ey * ey;
		}
	return 0.5 * sim->e0 * we * sim->dx[X] * sim->dx[Y];
}

static double
now(void)
{
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return (double) ts.tv_sec + 1e-9 * (double) ts.tv_nsec;
}

/* Timing mode: WARMUP untimed steps, the barrier through OUT_DIR, STEPS
 * timed steps. */
static int
time_steps(sim_t *sim, const char *dir, const char *spec)
{
	long long warm = 0, steps = 0, k, n = 0;
	char path[4096];
	FILE *f;
	int is;
	if(sscanf(spec, "%lld+%lld", &warm, &steps) != 2 || steps <= 0) die_msg("NSTEPS: WARMUP+STEPS");
	for(k = 0; k < warm; k++)
		if(sim_step(sim)) die_msg("sim_step failed");
	for(is = 0; is < (int) sim->nspecies; is++) n += sim->species[is].nparticles;
	snprintf(path, sizeof(path), "%s/ready.%d", dir, (int) getpid());
	if(!(f = fopen(path, "w"))) die_msg("cannot write ready file");
	fclose(f);
	snprintf(path, sizeof(path), "%s/go", dir);
	for(k = 0; access(path, F_OK) != 0; k++)
	{
		if(k > 6000000) die_msg("no go signal");   /* 10 min of 100 us naps */
		usleep(100);
	}
	double *t = malloc(sizeof(double) * (size_t) (steps + 1));
	if(!t) die_msg("out of memory");
	t[0] = now();
	for(k = 0; k < steps; k++)
	{
		if(sim_step(sim)) die_msg("sim_step failed");
		t[k + 1] = now();
	}
	snprintf(path, sizeof(path), "%s/times.%d", dir, (int) getpid());
	if(!(f = fopen(path, "wb"))) die_msg("cannot write times");
	int64_t n64 = n;
	wr(f, &n64, 8);
	wr(f, t, sizeof(double) * (size_t) (steps + 1));
	fclose(f);
	free(t);
	return 0;
}

int
main(int argc, char *argv[])
{
	config_t conf;
	sim_t *sim;
	FILE *f;
	int64_t is, nsteps, k;
	char path[4096];

	if(argc < 5) die_msg("usage: ref_harness CONF STATE_IN OUT_DIR NSTEPS [DUMP_STEPS...]");
	MPI_Init(&argc, &argv);
	config_init(&conf);
	if(config_read_file(&conf, argv[1]) != CONFIG_TRUE) die_msg("cannot read conf");
	sim = sim_init(&conf, 1);
	if(!sim) die_msg("sim_init failed");

	unsigned long long gseed = 0;
	double gv0 = 0.0, gvth = 0.0, gamp = 0.0;
	int timing = sscanf(argv[2], "two_stream:%llu:%lf:%lf:%lf", &gseed, &gv0, &gvth, &gamp) == 4;
	f = timing ? NULL : fopen(argv[2], "rb");
	if(!timing && !f) die_msg("cannot open state");
	for(is = 0; is < sim->nspecies; is++)
	{
		int64_t n, ic;
		double *x, *y, *ux, *uy;
		if(timing)
			n = sim->species[is].nparticles;
		else if(fread(&n, 8, 1, f) != 1)
			die_msg("short state");
		if(n != sim->species[is].nparticles) die_msg("particle count differs from conf");
		x = malloc(8 * (size_t) n); y = malloc(8 * (size_t) n);
		ux = malloc(8 * (size_t) n); uy = malloc(8 * (size_t) n);
		if(!x || !y || !ux || !uy) die_msg("out of memory");
		if(timing)
			seed_two_stream(gseed, (int) is, n, sim->L[X], sim->L[Y], gv0, gvth, gamp, x, y, ux, uy);
		else if(fread(x, 8, (size_t) n, f) != (size_t) n || fread(y, 8, (size_t) n, f) != (size_t) n
				|| fread(ux, 8, (size_t) n, f) != (size_t) n
				|| fread(uy, 8, (size_t) n, f) != (size_t) n)
			die_msg("short state");
		for(ic = 0; ic < sim->plasma.nchunks; ic++)
		{
			pblock_t *b;
			for(b = sim->plasma.chunks[ic].species[is].list.b; b; b = b->next)
			{
				int64_t q;
				for(q = 0; q < b->n; q++)
				{
					ppack_t *p = &b->p[q / MAX_VEC];
					int iv = (int) (q % MAX_VEC);
					int64_t id = p->i[iv];
					if(id < 0 || id >= n) die_msg("particle index out of range");
					p->r[X][iv] = x[id]; p->r[Y][iv] = y[id]; p->r[Z][iv] = 0.0;
					p->u[X][iv] = ux[id]; p->u[Y][iv] = uy[id]; p->u[Z][iv] = 0.0;
					p->E[X][iv] = 0.0; p->E[Y][iv] = 0.0; p->E[Z][iv] = 0.0;
				}
			}
		}
		free(x); free(y); free(ux); free(uy);
	}
	if(f) fclose(f);

	/* the pre-step on the injected state, sim.c:208-236 (iter is 0 here;
	 * the exchange tags only need to be consistent) */
	particle_comm_initial(sim);
	stage_field_rho(sim);
	stage_field_E(sim);
	if(timing)
		return time_steps(sim, argv[3], argv[4]);
	snprintf(path, sizeof(path), "%s/pre.bin", argv[3]);
	dump(sim, path);

	nsteps = atoll(argv[4]);
	snprintf(path, sizeof(path), "%s/energy.bin", argv[3]);
	FILE *fe = fopen(path, "wb");
	if(!fe) die_msg("cannot open energy file");
	for(k = 0; k < nsteps; k++)
	{
		int a;
		if(sim_step(sim)) die_msg("sim_step failed");
		double we = field_energy(sim);
		wr(fe, &we, 8);
		for(a = 5; a < argc; a++)
			if(atoll(argv[a]) == k + 1)
			{
				snprintf(path, sizeof(path), "%s/step%lld.bin", argv[3], (long long) (k + 1));
				dump(sim, path);
			}
	}
	fclose(fe);
	return 0;
}
