// bits_check.cpp -- checks cpic_gb300/csrc/cpic_bits.h against the FP64
// operations it replaces, on edge cases and random values (CPU test driven
// by tests/test_bits.py).  Prints the number of mismatches; 0 is a pass.
#include <cfenv>
#include <initializer_list>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../cpic_gb300/csrc/cpic_bits.h"

using namespace cpic::bits;

static long bad = 0, checked = 0, handled = 0;

static void check_split(double v, int lo_exp)
{
	long long hi, lo;
	checked++;
	if(!split_fixed(v, lo_exp, hi, lo))
		return;
	handled++;
	long long rhi = std::llrint(v);
	long long rlo = std::llrint((v - (double) rhi) * std::ldexp(1.0, lo_exp));
	if(hi != rhi || lo != rlo)
	{
		if(bad < 10)
			std::printf("split %.17g exp %d: %lld %lld, want %lld %lld\n", v, lo_exp, hi, lo, rhi, rlo);
		bad++;
	}
}

static void check_floor(double d)
{
	double f;
	int i;
	checked++;
	if(!floor_nonneg(d, f, i))
		return;
	handled++;
	double rf = std::floor(d);
	if(std::memcmp(&f, &rf, 8) != 0 || i != (int) rf)
	{
		if(bad < 10)
			std::printf("floor %.17g: %.17g %d\n", d, f, i);
		bad++;
	}
}

static void check_cmp(double d, double L)
{
	checked++;
	handled++;
	bool ok = ge_pos(d, L) == (d >= L) || std::isnan(d);
	ok = ok && (lt_zero(d) == (d < 0.0) || std::isnan(d));
	ok = ok && abs_gt(d, L) == (std::fabs(d) > L);
	ok = ok && is_finite(d) == (bool) std::isfinite(d);
	if(!ok)
	{
		if(bad < 10)
			std::printf("compare %.17g vs %.17g\n", d, L);
		bad++;
	}
}

int main()
{
	std::fesetround(FE_TONEAREST);
	std::mt19937_64 rng(12345);
	std::uniform_real_distribution<double> u01(0.0, 1.0);
	const int exps[] = {0, 1, 7, 20, 30, 31, 37, 40, 45, 52, 60};
	// exact ties and near-ties at many scales
	for(long long k = -4096; k <= 4096; k++)
		for(int sc = -8; sc <= 40; sc++)
		{
			double base = std::ldexp((double) k, sc);
			for(int e : exps)
			{
				check_split(base + 0.5, e);
				check_split(base - 0.5, e);
				check_split(std::nextafter(base + 0.5, 1e300), e);
				check_split(std::nextafter(base + 0.5, -1e300), e);
				check_split(base, e);
			}
		}
	// random magnitudes, both signs, and tiny values
	for(int t = 0; t < 4000000; t++)
	{
		double m = u01(rng) * 2.0 - 1.0;
		int sc = (int) (rng() % 130) - 70;
		double v = std::ldexp(m, sc);
		check_split(v, exps[t % 11]);
		check_split(v * 1e-250, exps[t % 11]);
		double d = std::fabs(std::ldexp(m, (int) (rng() % 40) - 8));
		check_floor(d);
	}
	for(double d : {0.0, -0.0, 0.5, 1.0, 1.5, 2.0, 2047.9999999999998, 2048.0, 3.0e9, 2147483647.0})
		check_floor(d);
	const double Ls[] = {6.283185307179586, 1.0, 32.0, 0.5, 1e-3, 12.566370614359172};
	for(double L : Ls)
	{
		for(double d : std::initializer_list<double>{0.0, -0.0, L, -L, std::nextafter(L, 0.0), std::nextafter(L, 1e300), 1e300,
				-1e300, (double) INFINITY, (double) -INFINITY, (double) NAN, (double) -NAN, 1e-310, -1e-310})
			check_cmp(d, L);
		for(int t = 0; t < 200000; t++)
			check_cmp(std::ldexp(u01(rng) * 2.0 - 1.0, (int) (rng() % 20) - 8) * L, L);
	}
	check_split(0.0, 30);
	check_split(-0.0, 30);
	// tile-row division: every n up to 4096 against t / n, for t over the
	// first rows, the last rows of a 4096-row grid and random indices
	for(uint32_t n = 1; n <= 4096; n++)
	{
		uint32_t mul;
		int sh;
		div_init(n, mul, sh);
		auto one = [&](uint32_t t) {
			checked++;
			handled++;
			if(div_q(t, mul, sh) != t / n)
			{
				if(bad < 10)
					std::printf("div %u / %u\n", t, n);
				bad++;
			}
		};
		for(uint32_t t = 0; t < 3 * n + 7; t++)
			one(t);
		for(uint32_t t = 4093 * n; t < 4096 * n; t++)
			one(t);
		for(int k = 0; k < 200; k++)
			one((uint32_t) (rng() % (1u << 30)));
		one((1u << 30) - 1);
	}
	std::printf("%ld mismatches of %ld handled (%ld checked)\n", bad, handled, checked);
	return bad != 0;
}
