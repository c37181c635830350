/*
 * cpic_oracle.c -- CPU restatement of cpic's 2D electrostatic PIC time step
 * (gather -> Boris push -> periodic re-bin -> CIC deposit -> FFT Poisson -> E).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle: only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it.
 * The product (cpic_gb300/) never links or calls it.
 *
 * Every routine follows the reference's FP64 arithmetic operation by
 * operation (same association, no contraction: build with
 * -ffp-contract=off) so that one-step particle positions are bit-exact with
 * the reference given identical fields.  Citations are file:line inside the
 * rodarima/cpic tree.
 *
 * Layout (same as the reference's mat_t views, MAT_XY = data[y*stride + x],
 * src/mat.h:75):
 *   rho : (ny + 2) rows x rstride = 2*(nx/2+1)   (row ny = ghost, row ny+1 =
 *         spill guard for a particle sitting exactly on y == L)
 *   phi : (ny + 3) rows x rstride, row 0 = north ghost (phi[-1])
 *   E   : (ny + 3) rows x nx  (row ny = ghost, two guard rows)
 *
 * Differences from the reference, all deliberate:
 *   - particles live in flat per-species arrays; the reference's re-bin
 *     (src/comm_plasma.c) only reorders particles, which changes the FP64
 *     summation order of the deposit and nothing else;
 *   - the deposit can run conflict-free (exact per-lane adds, the gate) or
 *     with the reference's lossy AVX2 lane update (src/simd_avx2.h:392-410);
 *   - the Poisson solve uses this file's own FFT instead of FFTW; parity
 *     with FFTW's rounding is unpinned.
 *   - a velocity above umax returns an error code instead of abort()
 *     (src/mover.c:97-137).
 */
#include <math.h>
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

#define ORC_MAX_SPECIES 8

typedef struct {
	double q, m;
	int64_t n;
	double *r[3];  /* r[X], r[Y], r[Z] */
	double *u[3];
	double *E[2];  /* field at the particle, as stored in ppack.E */
} orc_species_t;

typedef struct {
	int64_t nx, ny;
	double L[2], dx[2];
	double dt, e0, B[3];
	double umax[3];
	int64_t iter;
	int lossy_deposit;       /* 1 = reproduce the AVX2 lane-conflict loss */
	int64_t rstride;         /* 2*(nx/2+1) */
	double *rho, *phi, *E[2];
	double *G;               /* ny x (nx/2+1) Green's function */
	int nspecies;
	orc_species_t sp[ORC_MAX_SPECIES];
	int err;
} orc_t;

/* ------------------------------------------------------------------ FFT */

#include "orc_fft.h"

/* MFT Poisson solve, solver.c:465-509 (MFT_solve): r2c FFT of rho (rows
 * y, columns x: FFTW's n0 = ny, n1 = nx, solver.c:314-330), multiply by G
 * (MFT_kernel, solver.c:337-363, complex times real), c2r, divide by
 * nx*ny (MFT_normalize, solver.c:365-379).  rho and phi use row strides
 * rstride / pstride. */
static void
mft_solve(int64_t nx, int64_t ny, const double *G, const double *rho,
		int64_t rstride, double *phi, int64_t pstride)
{
	int64_t i, ix, iy, nh = nx / 2 + 1;
	double *sr = malloc(sizeof(double) * (size_t) (nh * ny));
	double *si = malloc(sizeof(double) * (size_t) (nh * ny));
	orc_rows_r2c(nx, ny, rho, rstride, sr, si);
	orc_cols(nx, ny, sr, si, -1);
	for(i = 0; i < nh * ny; i++)
	{
		sr[i] *= G[i];
		si[i] *= G[i];
	}
	orc_cols(nx, ny, sr, si, +1);
	orc_rows_c2r(nx, ny, sr, si, phi, pstride);
	for(iy = 0; iy < ny; iy++)
		for(ix = 0; ix < nx; ix++)
			phi[iy * pstride + ix] /= (double) (nx * ny);
	free(sr); free(si);
}

/* Green's function, solver.c:257-280 (MFT_init). */
static void
mft_green(int64_t nx, int64_t ny, double *G)
{
	int64_t ix, iy, nh = nx / 2 + 1;
	double cx = 2.0 * M_PI / nx;
	double cy = 2.0 * M_PI / ny;
	for(iy = 0; iy < ny; iy++)
		for(ix = 0; ix < nh; ix++)
		{
			if(ix == 0 && iy == 0)
				G[iy * nh + ix] = 0.0;
			else
				G[iy * nh + ix] = 1.0 /
					(2.0 * (cos(cx * ix) + cos(cy * iy)) - 4.0);
		}
}

/* ------------------------------------------------------- interpolation */

/* relative_position_grid, interpolate.c:38-66.  x0 is the field origin
 * (0 on a single rank).  Returns rel in [0,1] and the cell index the way
 * vf64_floor + vf64_to_vi64 produce it (simd_avx2.h:238-248). */
static inline double
rel_pos(double x0, double x, double dx, double idx, int64_t *i0)
{
	double block_delta = x - x0;
	double block_rel = block_delta * idx;
	double block_start = floor(block_rel);
	/* cvtpd_epi32 then zero-extension of the 32-bit lane */
	*i0 = (int64_t) (uint32_t) (int32_t) block_start;
	double grid_delta = block_delta - block_start * dx;
	return grid_delta * idx;
}

/* weights(), interpolate.c:77-100.  Quirk kept: the Y offset uses dx[X]
 * (interpolate.c:87-88).  w[0]=w00 w[1]=w01 w[2]=w10 w[3]=w11 as in
 * linear_interpolation, interpolate.c:11-32. */
static inline void
cic_weights(const orc_t *o, double x, double y, double idx, double idy,
		double w[4], int64_t i0[2])
{
	double rx = rel_pos(0.0, x, o->dx[0], idx, &i0[0]);
	double ry = rel_pos(0.0, y, o->dx[0], idy, &i0[1]);
	double delx = 1.0 - rx;
	double dely = 1.0 - ry;
	w[0] = delx * dely;
	w[1] = delx * ry;
	w[2] = rx * dely;
	w[3] = rx * ry;
}

/* interpolate_f2p, interpolate.c:102-155: the sum order is w00, w01, w10,
 * w11 over nodes (i0x,i0y) (i0x,i1y) (i1x,i0y) (i1x,i1y); i1x wraps
 * (vi64_remod), i1y uses the ghost row. */
static inline double
gather1(const orc_t *o, const double *mat, const double w[4], const int64_t i0[2])
{
	int64_t nx = o->nx;
	int64_t i1x = i0[0] + 1, i1y = i0[1] + 1;
	if(i1x >= nx) i1x -= nx;
	double v;
	v  = w[0] * mat[i0[1] * nx + i0[0]];
	v += w[1] * mat[i1y * nx + i0[0]];
	v += w[2] * mat[i0[1] * nx + i1x];
	v += w[3] * mat[i1y * nx + i1x];
	return v;
}

/* ------------------------------------------------------------- API */

orc_t *
orc_create(int64_t nx, int64_t ny, double Lx, double Ly, double dt, double e0,
		const double *B, int64_t plasma_chunks)
{
	orc_t *o = calloc(1, sizeof(*o));
	int64_t rows;
	if(!o) return NULL;
	o->nx = nx; o->ny = ny;
	o->L[0] = Lx; o->L[1] = Ly;
	/* sim_prepare, sim.c:171-175 */
	o->dx[0] = Lx / nx;
	o->dx[1] = Ly / ny;
	o->dt = dt; o->e0 = e0;
	o->B[0] = B[0]; o->B[1] = B[1]; o->B[2] = B[2];
	if(plasma_chunks < 1) plasma_chunks = 1;
	/* umax = chunksize * dx / dt, sim.c:198-200; Z has chunksize 1, dx 0 */
	o->umax[0] = (nx / plasma_chunks) * o->dx[0] / dt;
	o->umax[1] = ny * o->dx[1] / dt;
	o->umax[2] = 1 * 0.0 / dt;
	o->iter = -1;
	o->rstride = 2 * (nx / 2 + 1);
	rows = ny + 2;
	o->rho = calloc((size_t) (rows * o->rstride), sizeof(double));
	o->phi = calloc((size_t) ((ny + 3) * o->rstride), sizeof(double));
	o->E[0] = calloc((size_t) ((ny + 3) * nx), sizeof(double));
	o->E[1] = calloc((size_t) ((ny + 3) * nx), sizeof(double));
	o->G = malloc(sizeof(double) * (size_t) (ny * (nx / 2 + 1)));
	mft_green(nx, ny, o->G);
	return o;
}

void
orc_destroy(orc_t *o)
{
	int s, d;
	if(!o) return;
	for(s = 0; s < o->nspecies; s++)
	{
		for(d = 0; d < 3; d++) { free(o->sp[s].r[d]); free(o->sp[s].u[d]); }
		free(o->sp[s].E[0]); free(o->sp[s].E[1]);
	}
	free(o->rho); free(o->phi); free(o->E[0]); free(o->E[1]); free(o->G);
	free(o);
}

void orc_set_lossy_deposit(orc_t *o, int lossy) { o->lossy_deposit = lossy; }
int64_t orc_iter(const orc_t *o) { return o->iter; }
void orc_set_iter(orc_t *o, int64_t it) { o->iter = it; }
int orc_error(const orc_t *o) { return o->err; }

int
orc_add_species(orc_t *o, double q, double m, int64_t n,
		const double *x, const double *y,
		const double *ux, const double *uy, const double *uz)
{
	orc_species_t *s;
	int d;
	if(o->nspecies >= ORC_MAX_SPECIES) return -1;
	s = &o->sp[o->nspecies++];
	s->q = q; s->m = m; s->n = n;
	for(d = 0; d < 3; d++)
	{
		s->r[d] = calloc((size_t) (n > 0 ? n : 1), sizeof(double));
		s->u[d] = calloc((size_t) (n > 0 ? n : 1), sizeof(double));
	}
	s->E[0] = calloc((size_t) (n > 0 ? n : 1), sizeof(double));
	s->E[1] = calloc((size_t) (n > 0 ? n : 1), sizeof(double));
	memcpy(s->r[0], x, sizeof(double) * (size_t) n);
	memcpy(s->r[1], y, sizeof(double) * (size_t) n);
	memcpy(s->u[0], ux, sizeof(double) * (size_t) n);
	memcpy(s->u[1], uy, sizeof(double) * (size_t) n);
	if(uz) memcpy(s->u[2], uz, sizeof(double) * (size_t) n);
	return o->nspecies - 1;
}

int
orc_set_particles(orc_t *o, int is, const double *x, const double *y,
		const double *ux, const double *uy, const double *uz)
{
	orc_species_t *s = &o->sp[is];
	size_t b = sizeof(double) * (size_t) s->n;
	if(x) memcpy(s->r[0], x, b);
	if(y) memcpy(s->r[1], y, b);
	if(ux) memcpy(s->u[0], ux, b);
	if(uy) memcpy(s->u[1], uy, b);
	if(uz) memcpy(s->u[2], uz, b);
	return 0;
}

int
orc_get_particles(const orc_t *o, int is, double *x, double *y,
		double *ux, double *uy, double *uz, double *ex, double *ey)
{
	const orc_species_t *s = &o->sp[is];
	size_t b = sizeof(double) * (size_t) s->n;
	if(x) memcpy(x, s->r[0], b);
	if(y) memcpy(y, s->r[1], b);
	if(ux) memcpy(ux, s->u[0], b);
	if(uy) memcpy(uy, s->u[1], b);
	if(uz) memcpy(uz, s->u[2], b);
	if(ex) memcpy(ex, s->E[0], b);
	if(ey) memcpy(ey, s->E[1], b);
	return 0;
}

/* Field access: rho and phi as ny x nx (the view without padding/ghosts),
 * E as (ny+1) x nx including the south ghost row. */
void
orc_get_rho(const orc_t *o, double *out)
{
	int64_t iy;
	for(iy = 0; iy < o->ny; iy++)
		memcpy(out + iy * o->nx, o->rho + iy * o->rstride, sizeof(double) * (size_t) o->nx);
}

void
orc_set_rho(orc_t *o, const double *in)
{
	int64_t iy;
	for(iy = 0; iy < o->ny; iy++)
		memcpy(o->rho + iy * o->rstride, in + iy * o->nx, sizeof(double) * (size_t) o->nx);
}

void
orc_get_phi(const orc_t *o, double *out)
{
	int64_t iy;
	for(iy = 0; iy < o->ny; iy++)
		memcpy(out + iy * o->nx, o->phi + (iy + 1) * o->rstride, sizeof(double) * (size_t) o->nx);
}

void
orc_get_E(const orc_t *o, double *ex, double *ey)
{
	size_t b = sizeof(double) * (size_t) ((o->ny + 1) * o->nx);
	if(ex) memcpy(ex, o->E[0], b);
	if(ey) memcpy(ey, o->E[1], b);
}

void
orc_set_E(orc_t *o, const double *ex, const double *ey)
{
	size_t b = sizeof(double) * (size_t) ((o->ny + 1) * o->nx);
	if(ex) memcpy(o->E[0], ex, b);
	if(ey) memcpy(o->E[1], ey, b);
}

/* ------------------------------------------------------------ stages */

/* stage_field_E, field.c:450-501: solve (field_phi_solve, field.c:418),
 * exchange the phi ghosts with the single rank itself
 * (comm_phi_send/recv, comm_field.c:140-201: rows 0,1 -> south ghosts,
 * row ny-1 -> north ghost), then field_E_compute (field.c:358-416). */
int
orc_stage_field_E(orc_t *o)
{
	int64_t nx = o->nx, ny = o->ny, rs = o->rstride, ix, iy;
	double *phi = o->phi + rs;  /* view: row 0 = first interior row */
	double dx2, dy2;

	mft_solve(nx, ny, o->G, o->rho, rs, phi, rs);

	/* periodic ghosts of phi (whole padded rows are exchanged) */
	memcpy(phi + ny * rs, phi, sizeof(double) * (size_t) (2 * rs));
	memcpy(phi - rs, phi + (ny - 1) * rs, sizeof(double) * (size_t) rs);

	dx2 = 2 * o->dx[0];
	dy2 = 2 * o->dx[1];
	for(iy = 0; iy < ny + 1; iy++)
	{
		int64_t y0 = iy - 1, y1 = iy + 1;
		for(ix = 0; ix < nx; ix++)
		{
			int64_t x0 = (ix + nx - 1) % nx;
			int64_t x1 = (ix + 1) % nx;
			o->E[1][iy * nx + ix] = (phi[y0 * rs + ix] - phi[y1 * rs + ix]) / dy2;
			o->E[0][iy * nx + ix] = (phi[iy * rs + x0] - phi[iy * rs + x1]) / dx2;
		}
	}
	return 0;
}

/* stage_plasma_E -> interpolate_f2p_E, interpolate.c:349-404 and
 * particle.c:215-248. */
int
orc_stage_plasma_E(orc_t *o)
{
	int s;
	int64_t i;
	double idx = 1.0 / o->dx[0], idy = 1.0 / o->dx[1];
	for(s = 0; s < o->nspecies; s++)
	{
		orc_species_t *sp = &o->sp[s];
		for(i = 0; i < sp->n; i++)
		{
			double w[4];
			int64_t i0[2];
			cic_weights(o, sp->r[0][i], sp->r[1][i], idx, idy, w, i0);
			sp->E[0][i] = gather1(o, o->E[0], w, i0);
			cic_weights(o, sp->r[0][i], sp->r[1][i], idx, idy, w, i0);
			sp->E[1][i] = gather1(o, o->E[1], w, i0);
		}
	}
	return 0;
}

/* Boris push for one particle: boris_rotation (mover.c:22-70) with the
 * cross products of mover.c:14-20, check_velocity (mover.c:97-137), move
 * (mover.c:74-82), update_u (mover.c:85-93).  E[Z] is always 0. */
static inline int
boris1(const orc_t *o, double dtqm2, double dt, int set_r,
		double r[3], double u[3], const double E2[2])
{
	double t[3], s[3], sd[3], vm[3], vp[3], vpl[3], Ep[3];
	int d;
	Ep[0] = E2[0]; Ep[1] = E2[1]; Ep[2] = 0.0;
	for(d = 0; d < 3; d++)
	{
		sd[d] = 1.0;
		t[d] = o->B[d] * dtqm2;
		sd[d] += t[d] * t[d];
		vm[d] = u[d] + dtqm2 * Ep[d];
		s[d] = 2.0 * t[d] / sd[d];
	}
	vp[0] = vm[1] * t[2] - vm[2] * t[1];
	vp[1] = vm[2] * t[0] - vm[0] * t[2];
	vp[2] = vm[0] * t[1] - vm[1] * t[0];
	for(d = 0; d < 3; d++) vp[d] += vm[d];
	vpl[0] = vp[1] * s[2] - vp[2] * s[1];
	vpl[1] = vp[2] * s[0] - vp[0] * s[2];
	vpl[2] = vp[0] * s[1] - vp[1] * s[0];
	for(d = 0; d < 3; d++)
	{
		vpl[d] += vm[d];
		u[d] = vpl[d] + dtqm2 * Ep[d];
	}
	for(d = 0; d < 3; d++)
		if(fabs(u[d]) > o->umax[d])
			return -1;
	if(set_r)
		for(d = 0; d < 3; d++)
			r[d] += u[d] * dt;
	return 0;
}

/* periodic_boundary_ppack, comm_plasma.c:725-747: one wrap per call. */
static inline double
wrap1(double r, double L)
{
	if(r >= L) r -= L;
	else if(r < 0.0) r += L;
	return r;
}

/* stage_plasma_r, mover.c:331-362: chunk_update_r (mover.c:191-226) with
 * the iteration-0 backward half step, then comm_plasma(sim, 0)
 * (comm_plasma.c:1123): X then Y periodic wrap. */
int
orc_stage_plasma_r(orc_t *o)
{
	int s;
	int64_t i;
	double dt;
	int set_r;
	if(o->iter == 0) { dt = -o->dt / 2; set_r = 0; }
	else { dt = o->dt; set_r = 1; }
	for(s = 0; s < o->nspecies; s++)
	{
		orc_species_t *sp = &o->sp[s];
		/* dtqm2 = 0.5 * dt * q / m, mover.c:211 */
		double dtqm2 = 0.5 * dt * sp->q / sp->m;
		for(i = 0; i < sp->n; i++)
		{
			double r[3], u[3], E2[2];
			int d;
			for(d = 0; d < 3; d++) { r[d] = sp->r[d][i]; u[d] = sp->u[d][i]; }
			E2[0] = sp->E[0][i]; E2[1] = sp->E[1][i];
			if(boris1(o, dtqm2, dt, set_r, r, u, E2))
			{
				o->err = 1;
				return -1;
			}
			for(d = 0; d < 3; d++) { sp->r[d][i] = r[d]; sp->u[d][i] = u[d]; }
		}
		for(i = 0; i < sp->n; i++)
		{
			sp->r[0][i] = wrap1(sp->r[0][i], o->L[0]);
			sp->r[1][i] = wrap1(sp->r[1][i], o->L[1]);
		}
	}
	return 0;
}

/* Charge deposit: rho_reset (field.c:163-210: rows 0..ny, columns 0..nx-1),
 * interpolate_p2f_rho (interpolate.c:282-346) in packs of four particles,
 * each pack issuing vmat_add_xy for w00, w01, w10, w11 in turn
 * (interpolate.c:259-262), and the ghost fold of row ny into row 0
 * (comm_send/recv_ghost_rho, comm_field.c:52-136).  In lossy mode each
 * vmat_add_xy gathers the four old values first and stores lane by lane,
 * so colliding lanes lose all but the last update (simd_avx2.h:392-410). */
int
orc_stage_field_rho(orc_t *o)
{
	int64_t nx = o->nx, ny = o->ny, rs = o->rstride, ix, iy, i, s;
	double *rho = o->rho;
	double idx = 1.0 / o->dx[0], idy = 1.0 / o->dx[1];

	for(iy = 0; iy < ny + 1; iy++)
		for(ix = 0; ix < nx; ix++)
			rho[iy * rs + ix] = 0.0;

	for(s = 0; s < o->nspecies; s++)
	{
		orc_species_t *sp = &o->sp[s];
		double vq = -sp->q / o->e0;
		for(i = 0; i < sp->n; i += 4)
		{
			int64_t lanes = sp->n - i < 4 ? sp->n - i : 4, l, c;
			int64_t idxs[4][4];
			double val[4][4];
			for(l = 0; l < lanes; l++)
			{
				double w[4];
				int64_t i0[2], i1x, i1y;
				cic_weights(o, sp->r[0][i + l], sp->r[1][i + l], idx, idy, w, i0);
				i1x = i0[0] + 1; i1y = i0[1] + 1;
				if(i1x >= nx) i1x -= nx;
				idxs[0][l] = i0[1] * rs + i0[0];
				idxs[1][l] = i1y * rs + i0[0];
				idxs[2][l] = i0[1] * rs + i1x;
				idxs[3][l] = i1y * rs + i1x;
				for(c = 0; c < 4; c++) val[c][l] = w[c] * vq;
			}
			for(c = 0; c < 4; c++)
			{
				if(o->lossy_deposit)
				{
					double old[4];
					for(l = 0; l < lanes; l++) old[l] = rho[idxs[c][l]];
					for(l = 0; l < lanes; l++) rho[idxs[c][l]] = old[l] + val[c][l];
				}
				else
				{
					for(l = 0; l < lanes; l++) rho[idxs[c][l]] += val[c][l];
				}
			}
		}
	}

	/* ghost row ny folded into row 0 (self-send on a single rank) */
	for(ix = 0; ix < nx; ix++)
		rho[ix] += rho[ny * rs + ix];
	return 0;
}

/* sim_pre_step, sim.c:208-236: global re-bin (comm_plasma(sim, 1): on a
 * single rank only the Y wrap changes positions, comm_plasma.c:1087-1112),
 * stage_field_rho, stage_field_E. */
int
orc_pre_step(orc_t *o)
{
	int s;
	int64_t i;
	for(s = 0; s < o->nspecies; s++)
		for(i = 0; i < o->sp[s].n; i++)
			o->sp[s].r[1][i] = wrap1(o->sp[s].r[1][i], o->L[1]);
	orc_stage_field_rho(o);
	orc_stage_field_E(o);
	o->iter = 0;
	return 0;
}

/* sim_step, sim.c:481-581 (output, sampling and MPI_Bcast omitted). */
int
orc_step(orc_t *o)
{
	orc_stage_field_E(o);
	orc_stage_plasma_E(o);
	if(orc_stage_plasma_r(o)) return -1;
	orc_stage_field_rho(o);
	o->iter += 1;
	return 0;
}

int
orc_run(orc_t *o, int64_t nsteps)
{
	int64_t k;
	for(k = 0; k < nsteps; k++)
		if(orc_step(o)) return -1;
	return 0;
}

/* Diagnostics (the reference has none; sim.c:332-405 is compiled out):
 * field energy W_E = 0.5 e0 sum(Ex^2 + Ey^2) dx dy over the nx x ny nodes,
 * kinetic energy 0.5 sum m |u|^2, total charge sum(rho) dx dy and total
 * momentum sum m u.  out = {W_E, KE, Q, Px, Py}. */
void
orc_diag(const orc_t *o, double *out)
{
	int64_t ix, iy, i, nx = o->nx, ny = o->ny;
	int s;
	double we = 0.0, ke = 0.0, q = 0.0, px = 0.0, py = 0.0;
	for(iy = 0; iy < ny; iy++)
		for(ix = 0; ix < nx; ix++)
		{
			double ex = o->E[0][iy * nx + ix], ey = o->E[1][iy * nx + ix];
			we += ex * ex + ey * ey;
			q += o->rho[iy * o->rstride + ix];
		}
	we = 0.5 * o->e0 * we * o->dx[0] * o->dx[1];
	for(s = 0; s < o->nspecies; s++)
	{
		const orc_species_t *sp = &o->sp[s];
		double k = 0.0, sx = 0.0, sy = 0.0;
		for(i = 0; i < sp->n; i++)
		{
			k += sp->u[0][i] * sp->u[0][i] + sp->u[1][i] * sp->u[1][i]
				+ sp->u[2][i] * sp->u[2][i];
			sx += sp->u[0][i];
			sy += sp->u[1][i];
		}
		ke += 0.5 * sp->m * k;
		px += sp->m * sx;
		py += sp->m * sy;
	}
	out[0] = we;
	out[1] = ke;
	out[2] = q * o->dx[0] * o->dx[1];
	out[3] = px;
	out[4] = py;
}

/* Per-cell particle counts (cell = floor as in relative_position_grid),
 * ny x nx, int64. */
void
orc_cell_counts(const orc_t *o, int64_t *counts)
{
	int64_t i, nx = o->nx, ny = o->ny;
	int s;
	double idx = 1.0 / o->dx[0], idy = 1.0 / o->dx[1];
	memset(counts, 0, sizeof(int64_t) * (size_t) (nx * ny));
	for(s = 0; s < o->nspecies; s++)
		for(i = 0; i < o->sp[s].n; i++)
		{
			double w[4];
			int64_t i0[2];
			cic_weights(o, o->sp[s].r[0][i], o->sp[s].r[1][i], idx, idy, w, i0);
			if(i0[0] < nx && i0[1] < ny)
				counts[i0[1] * nx + i0[0]]++;
		}
}

/* Stand-alone pieces for known-answer tests. */
void
orc_weights(double x, double y, double x0, double y0, double dx, double dy,
		double *w, int64_t *i0)
{
	double idx = 1.0 / dx, idy = 1.0 / dy;
	double rx = rel_pos(x0, x, dx, idx, &i0[0]);
	double ry = rel_pos(y0, y, dx, idy, &i0[1]);
	w[0] = (1.0 - rx) * (1.0 - ry);
	w[1] = (1.0 - rx) * ry;
	w[2] = rx * (1.0 - ry);
	w[3] = rx * ry;
}

void
orc_poisson(int64_t nx, int64_t ny, const double *rho, double *phi)
{
	double *G = malloc(sizeof(double) * (size_t) (ny * (nx / 2 + 1)));
	mft_green(nx, ny, G);
	mft_solve(nx, ny, G, rho, nx, phi, nx);
	free(G);
}

/* ------------------------------------------------------- initial states
 *
 * The seeded two-stream and Maxwellian states of the benchmark workloads,
 * restated here so that the CPU legs of the benchmark build their inputs
 * without the product library.  The generator (seed_init.h) is the product's
 * init methods' (cpic_gb300/csrc/cpic_init.c); a CPU test checks the two bit
 * for bit. */

#include "seed_init.h"

/* Beams +v0 (first n/2) and -v0 with spread vth; x += amp sin(2 pi x / Lx),
 * wrapped into [0, Lx). */
void
orc_init_two_stream(uint64_t seed, int species, int64_t n, double Lx, double Ly,
		double v0, double vth, double amp, double *x, double *y, double *ux, double *uy)
{
	seed_two_stream(seed, species, n, Lx, Ly, v0, vth, amp, x, y, ux, uy);
}

/* Uniform positions, drifting 2D Maxwellian velocities. */
void
orc_init_maxwellian(uint64_t seed, int species, int64_t n, double Lx, double Ly,
		double vth, double driftx, double drifty, double *x, double *y, double *ux, double *uy)
{
	uint64_t s = 16u * (uint64_t) species;
	uint64_t bx = seed_stream(seed, s + 0), by = seed_stream(seed, s + 1);
	uint64_t bu = seed_stream(seed, s + 2), bv = seed_stream(seed, s + 3);
	int64_t i;
	for(i = 0; i < n; i++)
	{
		x[i] = seed_unif(bx, (uint64_t) i) * Lx;
		y[i] = seed_unif(by, (uint64_t) i) * Ly;
		ux[i] = driftx + vth * seed_gauss(bu, (uint64_t) i);
		uy[i] = drifty + vth * seed_gauss(bv, (uint64_t) i);
	}
}
