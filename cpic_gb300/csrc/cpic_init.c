/*
 * cpic_init.c -- seeded initial particle states for the two-stream,
 * Maxwellian and beam-plus-thermal set-ups.
 *
 * The reference initialises particles with glibc rand() through the
 * per-specie "init_method" table (src/particle.c:170-175: "random
 * position", "position delta").  Those methods cannot express drifting
 * Maxwellian beams or a sinusoidal density perturbation, so this file adds
 * them as further init methods with the same role.  Every draw is a pure
 * function of (seed, stream, particle index): a SplitMix64 counter
 * generator, so the state is reproducible in any order and in parallel.
 *
 * Host code only; no CUDA.
 */
#include <math.h>
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#include <stdint.h>
#include <string.h>

#include "../../include/cpic_gpu.h"

static inline uint64_t
mix64(uint64_t z)
{
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
	return z ^ (z >> 31);
}

#define GOLDEN 0x9E3779B97F4A7C15ULL

static inline uint64_t
stream_base(uint64_t seed, uint64_t stream)
{
	return mix64(seed * GOLDEN + mix64(stream + 0x632BE59BD9B4E019ULL));
}

/* i-th uniform in [0, 1) of a stream: the i-th output of a SplitMix64
 * sequence started at the stream's base state. */
static inline double
unif(uint64_t base, uint64_t i)
{
	return (double) (mix64(base + (i + 1) * GOLDEN) >> 11) * 0x1.0p-53;
}

/* Standard normal by Box-Muller from two uniforms of one stream. */
static inline double
gauss(uint64_t base, uint64_t i)
{
	double u1 = 1.0 - unif(base, 2 * i);   /* (0, 1] */
	double u2 = unif(base, 2 * i + 1);
	return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}

static inline double
wrap_pos(double x, double L)
{
	x = fmod(x, L);
	if(x < 0.0) x += L;
	if(x >= L) x -= L;
	return x;
}

CPIC_API void
cpic_uniform(uint64_t seed, uint64_t stream, int64_t n, double *out)
{
	uint64_t base = stream_base(seed, stream);
	int64_t i;
	#pragma omp parallel for schedule(static)
	for(i = 0; i < n; i++)
		out[i] = unif(base, (uint64_t) i);
}

CPIC_API void
cpic_normal(uint64_t seed, uint64_t stream, int64_t n, double *out)
{
	uint64_t base = stream_base(seed, stream);
	int64_t i;
	#pragma omp parallel for schedule(static)
	for(i = 0; i < n; i++)
		out[i] = gauss(base, (uint64_t) i);
}

/* Two counter-streaming beams: particles [0, n/2) drift at +v0, the rest at
 * -v0, both with a 2D Maxwellian spread vth; positions uniform in the box,
 * then x += amp * sin(2 pi x / Lx), wrapped into [0, Lx).  Streams
 * 16*species + {0,1,2,3} are x, y, vx, vy. */
CPIC_API void
cpic_init_two_stream(uint64_t seed, int species, int64_t n,
		double Lx, double Ly, double v0, double vth, double amp,
		double *x, double *y, double *ux, double *uy)
{
	uint64_t s = 16u * (uint64_t) species;
	uint64_t bx = stream_base(seed, s + 0), by = stream_base(seed, s + 1);
	uint64_t bu = stream_base(seed, s + 2), bv = stream_base(seed, s + 3);
	int64_t i, half = n / 2;
	#pragma omp parallel for schedule(static)
	for(i = 0; i < n; i++)
	{
		double px = unif(bx, (uint64_t) i) * Lx;
		double py = unif(by, (uint64_t) i) * Ly;
		if(amp != 0.0)
			px = wrap_pos(px + amp * sin(2.0 * M_PI * px / Lx), Lx);
		x[i] = px;
		y[i] = py;
		ux[i] = (i < half ? v0 : -v0) + (vth != 0.0 ? vth * gauss(bu, (uint64_t) i) : 0.0);
		uy[i] = vth != 0.0 ? vth * gauss(bv, (uint64_t) i) : 0.0;
	}
}

/* Uniform positions and a drifting 2D Maxwellian. */
CPIC_API void
cpic_init_maxwellian(uint64_t seed, int species, int64_t n,
		double Lx, double Ly, double vth, double driftx, double drifty,
		double *x, double *y, double *ux, double *uy)
{
	uint64_t s = 16u * (uint64_t) species;
	uint64_t bx = stream_base(seed, s + 0), by = stream_base(seed, s + 1);
	uint64_t bu = stream_base(seed, s + 2), bv = stream_base(seed, s + 3);
	int64_t i;
	#pragma omp parallel for schedule(static)
	for(i = 0; i < n; i++)
	{
		x[i] = unif(bx, (uint64_t) i) * Lx;
		y[i] = unif(by, (uint64_t) i) * Ly;
		ux[i] = driftx + vth * gauss(bu, (uint64_t) i);
		uy[i] = drifty + vth * gauss(bv, (uint64_t) i);
	}
}
