/*
 * simd_avx2.h (ORACLE-EXACT variant) -- the reference's own AVX2 layer with
 * one function replaced: vmat_add_xy adds lane by lane, so lanes of a
 * 4-particle pack that hit the same grid node all count.  The shipped
 * version gathers the four old values, adds and stores lane by lane, so the
 * last colliding lane overwrites the others (src/simd_avx2.h:392-410).
 * Everything else comes from the reference file itself, included by the
 * absolute path the build passes in ORC_REF_SIMD_AVX2.
 * TEST INFRASTRUCTURE ONLY.
 */
#pragma once
#define vmat_add_xy vmat_add_xy_as_shipped
#include ORC_REF_SIMD_AVX2
#undef vmat_add_xy

static inline void
vmat_add_xy(mat_t *m, vi64 ix, vi64 iy, vf64 x)
{
	vi64 idx = vmat_index_xy(m, ix, iy);
	size_t iv;
	for(iv = 0; iv < MAX_VEC; iv++)
		m->data[idx[iv]] += x[iv];
}
