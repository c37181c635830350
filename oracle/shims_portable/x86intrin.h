/*
 * x86intrin.h -- portable stand-in for the x86 intrinsics cpic's host code
 * uses (src/simd.h, src/simd_avx2.h, src/simd_common.h, src/solver.h:62-65),
 * so that the reference's sources build unchanged on hosts without AVX2
 * (the Arm host of the GPU) as well as on x86-64.
 *
 * TEST INFRASTRUCTURE.  Only the builds of the reference's own sources
 * (oracle/build_ref.py, tests/dropin_build.py) put this directory on the
 * include path, ahead of the system headers; the product never includes it.
 *
 * Every operation is written per lane with the IEEE semantics Intel documents
 * for the instruction: compares give all-ones / all-zero lanes, the FMA is a
 * single rounding (C99 fma), the double -> int32 conversion rounds with the
 * current rounding mode (round to nearest even by default, as MXCSR's
 * default), sqrt is correctly rounded and floor is exact.  The vector types
 * are GCC vector extensions of the same sizes as __m256d / __m256i /
 * __m128i, so the reference's arithmetic on them (a - b, casts between
 * them, m[i]) compiles as it does with the x86 headers.
 */
#ifndef CPIC_PORTABLE_X86INTRIN_H
#define CPIC_PORTABLE_X86INTRIN_H

#include <math.h>
#include <stdint.h>
#include <stdlib.h>     /* the x86 headers bring it in (mm_malloc.h); cpic relies on that */
#include <string.h>

/* mm_malloc.h declares it in the x86 headers, whatever the -std level */
extern int posix_memalign(void **memptr, size_t alignment, size_t size);

typedef double __m256d __attribute__((vector_size(32), aligned(32)));
typedef long long __m256i __attribute__((vector_size(32), aligned(32)));
typedef long long __m128i __attribute__((vector_size(16), aligned(16)));
typedef int __cpic_v4si __attribute__((vector_size(16)));

/* Compare predicates (the ordered, signalling forms cpic uses, plus their
 * quiet twins): value as in the AVX encoding. */
#define _CMP_EQ_OQ 0x00
#define _CMP_LT_OS 0x01
#define _CMP_LE_OS 0x02
#define _CMP_NEQ_UQ 0x04
#define _CMP_GE_OS 0x0d
#define _CMP_GT_OS 0x0e
#define _CMP_LT_OQ 0x11
#define _CMP_LE_OQ 0x12
#define _CMP_GE_OQ 0x1d
#define _CMP_GT_OQ 0x1e

#define _MM_HINT_T0 3
#define _mm_prefetch(p, hint) __builtin_prefetch((const void *) (p), 0, 3)

static inline int
__cpic_cmp1(double a, double b, int f)
{
	switch(f)
	{
		case _CMP_EQ_OQ: return a == b;
		case _CMP_LT_OS: case _CMP_LT_OQ: return a < b;
		case _CMP_LE_OS: case _CMP_LE_OQ: return a <= b;
		case _CMP_NEQ_UQ: return !(a == b);
		case _CMP_GE_OS: case _CMP_GE_OQ: return a >= b;
		case _CMP_GT_OS: case _CMP_GT_OQ: return a > b;
		default: return 0;
	}
}

static inline __m256d
_mm256_cmp_pd(__m256d a, __m256d b, const int f)
{
	__m256i m;
	for(int i = 0; i < 4; i++)
		m[i] = __cpic_cmp1(a[i], b[i], f) ? -1LL : 0LL;
	return (__m256d) m;
}

static inline __m256i
_mm256_cmpgt_epi64(__m256i a, __m256i b)
{
	__m256i m;
	for(int i = 0; i < 4; i++)
		m[i] = a[i] > b[i] ? -1LL : 0LL;
	return m;
}

static inline __m256i _mm256_and_si256(__m256i a, __m256i b) { return a & b; }
static inline __m256i _mm256_or_si256(__m256i a, __m256i b) { return a | b; }
static inline __m256i _mm256_xor_si256(__m256i a, __m256i b) { return a ^ b; }
static inline __m256i _mm256_andnot_si256(__m256i a, __m256i b) { return ~a & b; }

static inline __m256d
_mm256_and_pd(__m256d a, __m256d b)
{
	return (__m256d) ((__m256i) a & (__m256i) b);
}

static inline __m256d
_mm256_or_pd(__m256d a, __m256d b)
{
	return (__m256d) ((__m256i) a | (__m256i) b);
}

static inline __m256d
_mm256_xor_pd(__m256d a, __m256d b)
{
	return (__m256d) ((__m256i) a ^ (__m256i) b);
}

static inline __m256i
_mm256_set1_epi64x(long long x)
{
	__m256i v = {x, x, x, x};
	return v;
}

/* Arguments from the highest lane to the lowest, as the x86 header takes
 * them. */
static inline __m256i
_mm256_set_epi64x(long long e3, long long e2, long long e1, long long e0)
{
	__m256i v = {e0, e1, e2, e3};
	return v;
}

static inline __m256d
_mm256_set1_pd(double x)
{
	__m256d v = {x, x, x, x};
	return v;
}

static inline __m256d
_mm256_load_pd(const double *p)
{
	__m256d v;
	memcpy(&v, p, sizeof(v));
	return v;
}

static inline void
_mm256_store_pd(double *p, __m256d v)
{
	memcpy(p, &v, sizeof(v));
}

/* A non-temporal store is a hint; a plain store has the same effect. */
static inline void
_mm256_stream_pd(double *p, __m256d v)
{
	memcpy(p, &v, sizeof(v));
}

/* r[i] = *(double *) ((char *) base + index[i] * scale) */
static inline __m256d
_mm256_i64gather_pd(const double *base, __m256i index, const int scale)
{
	__m256d r;
	for(int i = 0; i < 4; i++)
		memcpy(&r[i], (const char *) base + index[i] * scale, sizeof(double));
	return r;
}

static inline __m256d
_mm256_sqrt_pd(__m256d a)
{
	__m256d r;
	for(int i = 0; i < 4; i++)
		r[i] = sqrt(a[i]);
	return r;
}

static inline __m256d
_mm256_floor_pd(__m256d a)
{
	__m256d r;
	for(int i = 0; i < 4; i++)
		r[i] = floor(a[i]);
	return r;
}

static inline __m256d
_mm256_fmadd_pd(__m256d a, __m256d b, __m256d c)
{
	__m256d r;
	for(int i = 0; i < 4; i++)
		r[i] = fma(a[i], b[i], c[i]);
	return r;
}

/* Four doubles -> four int32 in the low 128 bits, rounded with the current
 * rounding mode; out of range gives INT32_MIN, the x86 "integer
 * indefinite" value. */
static inline __m128i
_mm256_cvtpd_epi32(__m256d a)
{
	__cpic_v4si r;
	for(int i = 0; i < 4; i++)
	{
		double v = nearbyint(a[i]);
		r[i] = (v >= -2147483648.0 && v < 2147483648.0) ? (int) v : (int) 0x80000000u;
	}
	return (__m128i) r;
}

/* Four unsigned int32 (low 128 bits) zero-extended to four int64. */
static inline __m256i
_mm256_cvtepu32_epi64(__m128i a)
{
	__cpic_v4si v = (__cpic_v4si) a;
	__m256i r;
	for(int i = 0; i < 4; i++)
		r[i] = (long long) (unsigned int) v[i];
	return r;
}

static inline int
_mm256_movemask_pd(__m256d a)
{
	__m256i v = (__m256i) a;
	int m = 0;
	for(int i = 0; i < 4; i++)
		m |= (int) (((unsigned long long) v[i] >> 63) & 1u) << i;
	return m;
}

/* MXCSR: the reference reads it before each solve and restores its
 * desired value (src/solver.c:470-472).  Without SSE there is no such
 * register; the stand-in reports the x86 power-on value (all exceptions
 * masked, round to nearest) and ignores writes. */
#define __builtin_ia32_stmxcsr() (0x1f80u)
#define __builtin_ia32_ldmxcsr(v) ((void) (v))

#endif /* CPIC_PORTABLE_X86INTRIN_H */
