// cpic_bits.h -- exact FP64 conversions done with integer operations on the
// bits of a double.
//
// The FP64 form computes, per particle, the floor of its position in cell
// units (converted to an int cell index) and splits each of its four
// fixed-point deposit values v into hi = rn(v) (the nearest integer, ties to
// even) and lo = rn((v - hi) * 2^m).  In FP64 arithmetic these are FRND,
// F2I, I2F, DADD, DMUL and F2I instructions, all on the FP64 pipe, which is
// narrow on this GPU (about 1.7 instructions per clock per SM, against 64
// for 32-bit integer operations) and is what bounds the FP64 form.  The
// functions below give the same results exactly, bit for bit, from the IEEE
// representation with integer shifts, masks and adds.  They are plain C++
// (host and device), so a CPU test checks them against the FP64 operations
// on edge cases and random values.
#pragma once
#include <climits>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define CPIC_HD __host__ __device__ __forceinline__
#else
#define CPIC_HD inline
#endif

namespace cpic {
namespace bits {

CPIC_HD uint64_t to_bits(double d)
{
#ifdef __CUDA_ARCH__
	return (uint64_t) __double_as_longlong(d);
#else
	uint64_t b;
	std::memcpy(&b, &d, 8);
	return b;
#endif
}

CPIC_HD double from_bits(uint64_t b)
{
#ifdef __CUDA_ARCH__
	return __longlong_as_double((long long) b);
#else
	double d;
	std::memcpy(&d, &b, 8);
	return d;
#endif
}

// floor(d) and its value as an int, for 0 <= d < 2^31 (true when the
// result is false: the caller then uses the FP64 instructions).  +0.0 and
// every d in [0, 1) give +0.0 and 0.
CPIC_HD bool floor_nonneg(double d, double &f, int &i)
{
	const uint64_t b = to_bits(d);
	if(b >> 63)
		return false;                       // negative (or -0.0): not handled
	const int e = (int) ((b >> 52) & 0x7ff) - 1023;
	if(e < 0)
	{
		f = 0.0;
		i = 0;
		return true;
	}
	if(e > 30)
		return false;                       // >= 2^31, or Inf / NaN
	const uint64_t m = (b & 0xfffffffffffffull) | (1ull << 52);
	const int sh = 52 - e;                  // 22 .. 52 fractional bits
	f = from_bits(b & ~((1ull << sh) - 1ull));
	i = (int) (m >> sh);
	return true;
}

// The compares of the periodic wrap and of the velocity check, from the
// bits (positive doubles order like their bit patterns read as integers).
// Each gives the IEEE compare's result for every finite or infinite d; for a
// NaN d the caller's result is NaN either way and is reported as such.

// d >= L, for a finite L > 0
CPIC_HD bool ge_pos(double d, double L)
{
	return (int64_t) to_bits(d) >= (int64_t) to_bits(L);
}

// d < 0.0 (false for -0.0)
CPIC_HD bool lt_zero(double d)
{
	const int64_t b = (int64_t) to_bits(d);
	return b < 0 && b != INT64_MIN;
}

// |d| > u, for a finite u >= 0 (false for a NaN d, as the IEEE compare)
CPIC_HD bool abs_gt(double d, double u)
{
	const uint64_t a = to_bits(d) & 0x7fffffffffffffffull;
	return a > to_bits(u) && a <= 0x7ff0000000000000ull;
}

// d is neither infinite nor NaN
CPIC_HD bool is_finite(double d)
{
	return (to_bits(d) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull;
}

// Division of a tile index by the number of tiles per row without a divide
// instruction: q = t / n = (t * mul) >> sh (a 32 x 32 -> 64-bit product and
// a shift), exact for every t < 2^30 and n in [1, 2^30).  With D = 2n,
// c = ceil(log2 D) and mul = ceil(2^(31+c) / D) < 2^32: t * mul / 2^(30+c)
// = 2t * mul / 2^(31+c) = t/n + 2t e / (D 2^(31+c)) with e = mul D -
// 2^(31+c) < D <= 2^c, an excess below 1/n for 2t < 2^31.  For a power of
// two n, mul = 2^31 and the result is t >> log2 n.
CPIC_HD void div_init(uint32_t n, uint32_t &mul, int &sh)
{
	const uint64_t D = 2ull * n;
	int c = 0;
	while((1ull << c) < D)
		c++;
	mul = (uint32_t) (((1ull << (31 + c)) + D - 1) / D);
	sh = 30 + c;
}

CPIC_HD uint32_t div_q(uint32_t t, uint32_t mul, int sh)
{
	return (uint32_t) (((uint64_t) t * mul) >> sh);
}

// mag / 2^k rounded to the nearest integer, ties to even, for k >= 0.
CPIC_HD uint64_t rshift_rne(uint64_t mag, int k)
{
	if(k == 0)
		return mag;
	if(k > 64)
		return 0;                           // mag < 2^64 <= half of 2^k
	const uint64_t q = k == 64 ? 0 : mag >> k;
	const uint64_t r = k == 64 ? mag : mag & ((1ull << k) - 1ull);
	const uint64_t half = 1ull << (k - 1);
	return q + ((r > half || (r == half && (q & 1ull))) ? 1ull : 0ull);
}

// hi = rn(v), lo = rn((v - hi) * 2^lo_exp) for a finite v with |v| < 2^62
// (false otherwise: the caller then uses the FP64 instructions); rn rounds
// to the nearest integer, ties to even, as __double2ll_rn does.  v - hi is
// exact in FP64 and so is its product by a power of two, so lo's only
// rounding is the final one, which this reproduces on the integer
// fraction.
CPIC_HD bool split_fixed(double v, int lo_exp, long long &hi, long long &lo)
{
	const uint64_t b = to_bits(v);
	const bool neg = (b >> 63) != 0;
	const int E = (int) ((b >> 52) & 0x7ff);
	if(E == 0x7ff)
		return false;                       // Inf / NaN
	if(E == 0)
	{
		if((b & 0xfffffffffffffull) != 0)
			return false;                       // subnormal: not handled
		hi = 0;
		lo = 0;
		return true;
	}
	const int e = E - 1023;
	if(e >= 62)
		return false;
	const uint64_t m = (b & 0xfffffffffffffull) | (1ull << 52);
	const int sh = 52 - e;                  // fractional bits of |v| = m 2^-sh
	uint64_t him, lom;
	if(sh <= 0)
	{
		him = m << (-sh);                       // an integer: nothing below
		lom = 0;
		hi = neg ? -(long long) him : (long long) him;
		lo = 0;
		return true;
	}
	// |v| = m 2^-sh; its integer part q, remainder r < 2^sh (sh up to 1074:
	// beyond 63 fractional bits q is 0 and r is m itself)
	const uint64_t q = sh >= 64 ? 0 : m >> sh;
	const bool r_all = sh >= 64;
	const uint64_t r = r_all ? m : m & ((1ull << sh) - 1ull);
	// round half to even: up when r > 2^(sh-1), or equal and q odd
	bool up;
	if(sh > 64)
		up = false;                             // r = m < 2^53 < 2^(sh-1)
	else
	{
		const uint64_t half = 1ull << (sh - 1);
		up = r > half || (r == half && (q & 1ull));
	}
	him = q + (up ? 1ull : 0ull);
	// |v| - him = f 2^-sh, f = r - up 2^sh (signed; |f| <= 2^(sh-1));
	// lo = rn(f 2^(lo_exp - sh)), symmetric in the sign of f
	bool fneg;
	uint64_t fmag;
	if(!up)
	{
		fneg = false;
		fmag = r;
	}
	else
	{
		fneg = true;                            // r - 2^sh < 0 (sh <= 64 here)
		fmag = sh == 64 ? (uint64_t) 0 - r : (1ull << sh) - r;
	}
	const int k = sh - lo_exp;              // right shift of the fraction
	if(k <= 0)
	{
		if(-k >= 64 || (fmag >> (63 + k)) != 0)
			return false;                       // would not fit in 63 bits
		lom = fmag << (-k);
	}
	else
		lom = rshift_rne(fmag, k);
	const bool lneg = neg != fneg;
	hi = neg ? -(long long) him : (long long) him;
	lo = lneg ? -(long long) lom : (long long) lom;
	return true;
}

} // namespace bits
} // namespace cpic
