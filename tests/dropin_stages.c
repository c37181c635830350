/*
 * dropin_stages.c -- runs a .conf through the drop-in sim layer
 * (cpic_gb300/dropin/sim_gpu.c) and dumps the host views it leaves.
 * TEST INFRASTRUCTURE.
 *
 * usage: dropin_stages CONF NSTEPS MODE OUT
 *   MODE run     sim_run (cycles = NSTEPS in the conf)
 *        step    NSTEPS calls of sim_step
 *        stages  NSTEPS times the reference's stage sequence called one by
 *                one, as sim_step does it (sim.c:481-581): stage_field_E,
 *                output_fields, stage_plasma_E, stage_plasma_r,
 *                stage_field_rho, then iter + 1
 *
 * OUT: int64 nspecies; per species int64 n, then n records of int64 id and
 * six doubles x, y, ux, uy, Ex, Ey (plist order); then int64 nx, ny and the
 * ny x nx views of rho, phi, E_x, E_y.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <libconfig.h>
#include <mpi.h>

#include "sim.h"
#include "def.h"
#include "comm.h"
#include "field.h"
#include "output.h"
#include "particle.h"

static void
w64(FILE *f, int64_t v)
{
	fwrite(&v, sizeof(v), 1, f);
}

static void
wview(FILE *f, mat_t *m, i64 nx, i64 ny)
{
	for(i64 iy = 0; iy < ny; iy++)
		for(i64 ix = 0; ix < nx; ix++)
		{
			double v = MAT_XY(m, ix, iy);
			fwrite(&v, sizeof(v), 1, f);
		}
}

static int
dump(sim_t *sim, const char *path)
{
	FILE *f = fopen(path, "wb");
	if(!f) return 1;
	w64(f, sim->nspecies);
	for(i64 is = 0; is < sim->nspecies; is++)
	{
		int64_t n = 0;
		for(i64 ic = 0; ic < sim->plasma.nchunks; ic++)
			for(pblock_t *b = sim->plasma.chunks[ic].species[is].list.b; b; b = b->next)
				n += b->n;
		w64(f, n);
		for(i64 ic = 0; ic < sim->plasma.nchunks; ic++)
			for(pblock_t *b = sim->plasma.chunks[ic].species[is].list.b; b; b = b->next)
				for(i64 j = 0; j < b->n; j++)
				{
					ppack_t *p = &b->p[j / MAX_VEC];
					int iv = (int) (j % MAX_VEC);
					double v[6] = {p->r[X][iv], p->r[Y][iv], p->u[X][iv], p->u[Y][iv],
						p->E[X][iv], p->E[Y][iv]};
					w64(f, p->i[iv]);
					fwrite(v, sizeof(double), 6, f);
				}
	}
	i64 nx = sim->ntpoints[X], ny = sim->ntpoints[Y];
	w64(f, nx);
	w64(f, ny);
	wview(f, sim->field.rho, nx, ny);
	wview(f, sim->field.phi, nx, ny);
	wview(f, sim->field.E[X], nx, ny);
	wview(f, sim->field.E[Y], nx, ny);
	return fclose(f) != 0;
}

int
main(int argc, char *argv[])
{
	config_t conf;
	sim_t *sim;

	if(argc != 5)
	{
		fprintf(stderr, "usage: %s CONF NSTEPS run|step|stages OUT\n", argv[0]);
		return 2;
	}
	long nsteps = atol(argv[2]);
	const char *mode = argv[3];
	MPI_Init(NULL, NULL);
	config_init(&conf);
	if(config_read_file(&conf, argv[1]) == CONFIG_FALSE)
	{
		fprintf(stderr, "cannot read %s\n", argv[1]);
		return 2;
	}
	if(!(sim = sim_init(&conf, 1)))
	{
		fprintf(stderr, "sim_init failed\n");
		return 1;
	}
	if(!strcmp(mode, "run"))
	{
		if(sim_run(sim))
			return 1;
	}
	else if(!strcmp(mode, "step"))
	{
		for(long k = 0; k < nsteps; k++)
			if(sim_step(sim))
				return 1;
	}
	else if(!strcmp(mode, "stages"))
	{
		for(long k = 0; k < nsteps; k++)
		{
			if(stage_field_E(sim))
				return 1;
			if(output_fields(sim))
				return 1;
			stage_plasma_E(sim);
			stage_plasma_r(sim);
			stage_field_rho(sim);
			sim->iter += 1;
			sim->t = sim->iter * sim->dt;
		}
		/* the void stages report a failure through the next call */
		if(comm_plasma(sim, 0))
			return 1;
	}
	else
		return 2;
	if(dump(sim, argv[4]))
		return 1;
	MPI_Finalize();
	return 0;
}
