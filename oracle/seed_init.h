/*
 * seed_init.h -- the seeded initial states of the benchmark workloads, for
 * the CPU side: the oracle (cpic_oracle.c) and the reference harness
 * (ref_harness.c), so that neither needs the product library to build its
 * input.  TEST INFRASTRUCTURE.
 *
 * Same generator as the product's init methods (cpic_gb300/csrc/cpic_init.c):
 * every draw is the SplitMix64 finaliser of (stream base + (i + 1) * golden
 * ratio), the top 53 bits scaled to [0, 1); normals by Box-Muller from draws
 * 2i and 2i+1 of a stream; streams 16 * species + {0, 1, 2, 3} are x, y, ux,
 * uy.  tests/test_abi.py checks the oracle's arrays against the product's bit
 * for bit.
 */
#ifndef CPIC_SEED_INIT_H
#define CPIC_SEED_INIT_H

#include <math.h>
#include <stdint.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static inline uint64_t
seed_mix64(uint64_t z)
{
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
	return z ^ (z >> 31);
}

#define SEED_GOLDEN 0x9E3779B97F4A7C15ULL

static inline uint64_t
seed_stream(uint64_t seed, uint64_t stream)
{
	return seed_mix64(seed * SEED_GOLDEN + seed_mix64(stream + 0x632BE59BD9B4E019ULL));
}

static inline double
seed_unif(uint64_t base, uint64_t i)
{
	return (double) (seed_mix64(base + (i + 1) * SEED_GOLDEN) >> 11) * 0x1.0p-53;
}

static inline double
seed_gauss(uint64_t base, uint64_t i)
{
	double u1 = 1.0 - seed_unif(base, 2 * i);
	double u2 = seed_unif(base, 2 * i + 1);
	return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}

/* Beams +v0 (first n/2) and -v0 with spread vth; x += amp sin(2 pi x / Lx),
 * wrapped into [0, Lx). */
static inline void
seed_two_stream(uint64_t seed, int species, int64_t n, double Lx, double Ly,
		double v0, double vth, double amp, double *x, double *y, double *ux, double *uy)
{
	uint64_t s = 16u * (uint64_t) species;
	uint64_t bx = seed_stream(seed, s + 0), by = seed_stream(seed, s + 1);
	uint64_t bu = seed_stream(seed, s + 2), bv = seed_stream(seed, s + 3);
	int64_t i, half = n / 2;
	for(i = 0; i < n; i++)
	{
		double px = seed_unif(bx, (uint64_t) i) * Lx;
		double py = seed_unif(by, (uint64_t) i) * Ly;
		if(amp != 0.0)
		{
			px = fmod(px + amp * sin(2.0 * M_PI * px / Lx), Lx);
			if(px < 0.0) px += Lx;
			if(px >= Lx) px -= Lx;
		}
		x[i] = px;
		y[i] = py;
		ux[i] = (i < half ? v0 : -v0) + (vth != 0.0 ? vth * seed_gauss(bu, (uint64_t) i) : 0.0);
		uy[i] = vth != 0.0 ? vth * seed_gauss(bv, (uint64_t) i) : 0.0;
	}
}

#endif /* CPIC_SEED_INIT_H */
