// cpic_mixed.cu -- mixed-precision form: int32 cell + FP32 offset, FP32
// velocity, E and FFT; charge reduction in 64-bit fixed point, k=0 removal
// in FP64.  FMA contraction is allowed here.
#include <algorithm>
#include "cpic_common.cuh"
#include "cpic_push.cuh"
#include "cpic_fft.cuh"

namespace cpic {

// E = -grad(phi), FP32, periodic (field_E_compute, src/field.c:358-416),
// stored as (Ex, Ey) pairs for the per-tile shared-memory stage.  Rows
// over blockIdx.y, so no index is divided.
__global__ void k_E_mix(Grid g, const float *phi, float2 *E)
{
	// four nodes of one row per thread (nx a multiple of 4): one float4 of
	// phi from each of the three rows, the two x neighbours outside it,
	// two float4 stores of E
	const int nq = g.nx >> 2;
	const float rdx2 = (float) (1.0 / (2 * g.dx)), rdy2 = (float) (1.0 / (2 * g.dy));
	for(int iy = blockIdx.y; iy < g.ny; iy += gridDim.y)
	{
		const int y0 = iy == 0 ? g.ny - 1 : iy - 1;
		const int y1 = iy + 1 == g.ny ? 0 : iy + 1;
		const float *r = phi + (int64_t) iy * g.nx;
		const float *ru = phi + (int64_t) y0 * g.nx;
		const float *rd = phi + (int64_t) y1 * g.nx;
		for(int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x)
		{
			const int x = q << 2;
			const float4 c = *reinterpret_cast<const float4 *>(r + x);
			const float4 u = *reinterpret_cast<const float4 *>(ru + x);
			const float4 d = *reinterpret_cast<const float4 *>(rd + x);
			const float l = r[x == 0 ? g.nx - 1 : x - 1], rr = r[x + 4 == g.nx ? 0 : x + 4];
			float4 e0, e1;
			e0.x = (l - c.y) * rdx2;   e0.y = (u.x - d.x) * rdy2;
			e0.z = (c.x - c.z) * rdx2; e0.w = (u.y - d.y) * rdy2;
			e1.x = (c.y - c.w) * rdx2; e1.y = (u.z - d.z) * rdy2;
			e1.z = (c.z - rr) * rdx2;  e1.w = (u.w - d.w) * rdy2;
			float4 *o = reinterpret_cast<float4 *>(E + (int64_t) iy * g.nx + x);
			o[0] = e0;
			o[1] = e1;
		}
	}
}

// The same for any nx: one node per thread.
__global__ void k_E_mix_any(Grid g, const float *phi, float2 *E)
{
	const float rdx2 = (float) (1.0 / (2 * g.dx)), rdy2 = (float) (1.0 / (2 * g.dy));
	for(int iy = blockIdx.y; iy < g.ny; iy += gridDim.y)
	{
		const int y0 = iy == 0 ? g.ny - 1 : iy - 1;
		const int y1 = iy + 1 == g.ny ? 0 : iy + 1;
		const float *r = phi + (int64_t) iy * g.nx;
		for(int x = blockIdx.x * blockDim.x + threadIdx.x; x < g.nx; x += gridDim.x * blockDim.x)
		{
			const int xm = x == 0 ? g.nx - 1 : x - 1, xp = x + 1 == g.nx ? 0 : x + 1;
			float2 e;
			e.x = (r[xm] - r[xp]) * rdx2;
			e.y = (phi[(int64_t) y0 * g.nx + x] - phi[(int64_t) y1 * g.nx + x]) * rdy2;
			E[(int64_t) iy * g.nx + x] = e;
		}
	}
}

void launch_E_mix(const Grid &g, const float *phi, float2 *E, cudaStream_t s)
{
	const bool quads = g.nx % 4 == 0;
	const int per_row = quads ? g.nx >> 2 : g.nx;
	dim3 grid((per_row + 255) / 256, 1);
	grid.y = (unsigned) std::min(g.ny, std::max(1, 8 * 152 / (int) grid.x));
	if(quads) k_E_mix<<<grid, 256, 0, s>>>(g, phi, E);
	else k_E_mix_any<<<grid, 256, 0, s>>>(g, phi, E);
}

// E at every particle of a mixed store, by particle id (ids required).
__global__ void k_gather_mix(Grid g, StoreMix st, const int64_t *base, const int32_t *cnt,
		const float2 *E, double *ex_out, double *ey_out)
{
	int t = blockIdx.x;
	int n = cnt[t];
	int64_t b = base[t];
	for(int i = threadIdx.x; i < n; i += blockDim.x)
	{
		int c = st.cell[b + i];
		int cx = c & ((1 << g.lcx) - 1), cy = c >> g.lcx;
		int x1 = cx + 1 == g.nx ? 0 : cx + 1;
		int y1 = cy + 1 == g.ny ? 0 : cy + 1;
		const float4 v = st.ou[b + i];
		float ox = v.x, oy = v.y;
		float dxo = 1.0f - ox, dyo = 1.0f - oy;
		float2 e00 = E[(int64_t) cy * g.nx + cx], e01 = E[(int64_t) y1 * g.nx + cx];
		float2 e10 = E[(int64_t) cy * g.nx + x1], e11 = E[(int64_t) y1 * g.nx + x1];
		float ex = dxo * dyo * e00.x + dxo * oy * e01.x + ox * dyo * e10.x + ox * oy * e11.x;
		float ey = dxo * dyo * e00.y + dxo * oy * e01.y + ox * dyo * e10.y + ox * oy * e11.y;
		int id = st.id ? st.id[b + i] : (int) (b + i);
		ex_out[id] = ex;
		ey_out[id] = ey;
	}
}

void launch_gather_mix_tiles(const Grid &g, const StoreMix &st, const int64_t *base,
		const int32_t *cnt, int ntiles, const float2 *E, double *ex_out, double *ey_out,
		cudaStream_t s)
{
	k_gather_mix<<<ntiles, 256, 0, s>>>(g, st, base, cnt, E, ex_out, ey_out);
}

static PerDeviceOnce g_push_mix_once, g_poisson_mix_once;

// The fused kernel's instance: register-capped (Mix::kHiBlocks resident
// blocks) or not, store with or without ids, P particles per thread, grid
// of powers of two or not (the cell wrap).
template <int P, bool G>
static const void *push_mix_fn_pg(bool hi, bool ids)
{
	if(hi)
		return ids ? (const void *) k_push<Mix, Mix::kHiBlocks, true, P, G>
			: (const void *) k_push<Mix, Mix::kHiBlocks, false, P, G>;
	return ids ? (const void *) k_push<Mix, Mix::kMinBlocks, true, P, G>
		: (const void *) k_push<Mix, Mix::kMinBlocks, false, P, G>;
}

template <int P>
static const void *push_mix_fn_p(bool hi, bool ids, bool gp2)
{
	return gp2 ? push_mix_fn_pg<P, true>(hi, ids) : push_mix_fn_pg<P, false>(hi, ids);
}

static const void *push_mix_fn(bool hi, bool ids, int P, bool gp2)
{
	return P == 1 ? push_mix_fn_p<1>(hi, ids, gp2) : P == 4 ? push_mix_fn_p<4>(hi, ids, gp2)
		: push_mix_fn_p<2>(hi, ids, gp2);
}

static cudaError_t push_mix_attrs()
{
	return g_push_mix_once.run([] {
		cudaError_t e = cudaSuccess;
		for(int P : kPPTChoices)
			for(int hi = 0; hi < 2 && e == cudaSuccess; hi++)
				for(int ids = 0; ids < 2 && e == cudaSuccess; ids++)
					for(int gp2 = 0; gp2 < 2 && e == cudaSuccess; gp2++)
						e = set_max_dyn_smem({push_mix_fn(hi != 0, ids != 0, P, gp2 != 0)},
								200 * 1024, true);
		return e;
	});
}

// Whether the register-capped instance of the fused kernel reaches its
// Mix::kHiBlocks resident blocks per SM with this much dynamic shared
// memory (else the unconstrained instance runs).  The ids and no-ids
// instances of a block count use the same registers within a few.
static bool push_mix_hi(size_t smem, bool ids, int ppt, bool gp2)
{
	if(push_mix_attrs() != cudaSuccess)
		return false;
	int hi = 0;
	cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&hi,
			push_mix_fn(true, ids, ppt, gp2), kPushThreads, smem);
	return e == cudaSuccess && hi >= Mix::kHiBlocks;
}

int push_mix_blocks_per_sm(size_t smem, bool ids, int ppt, bool gp2)
{
	if(!ppt_supported(ppt))
		return 0;
	if(push_mix_hi(smem, ids, ppt, gp2))
		return Mix::kHiBlocks;
	int lo = 0;
	cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&lo,
			push_mix_fn(false, ids, ppt, gp2), kPushThreads, smem);
	return e == cudaSuccess ? lo : 0;
}

template <int P, bool G>
static void launch_push_mix_pg(const PushArgs &b, int ntiles, size_t smem, bool hi, bool ids,
		cudaStream_t s)
{
	if(ids)
	{
		if(hi) k_push<Mix, Mix::kHiBlocks, true, P, G><<<ntiles, kPushThreads, smem, s>>>(b);
		else k_push<Mix, Mix::kMinBlocks, true, P, G><<<ntiles, kPushThreads, smem, s>>>(b);
	}
	else
	{
		if(hi) k_push<Mix, Mix::kHiBlocks, false, P, G><<<ntiles, kPushThreads, smem, s>>>(b);
		else k_push<Mix, Mix::kMinBlocks, false, P, G><<<ntiles, kPushThreads, smem, s>>>(b);
	}
}

template <int P>
static void launch_push_mix_p(const PushArgs &b, int ntiles, size_t smem, bool hi, bool ids,
		cudaStream_t s)
{
	if(b.g.pow2) launch_push_mix_pg<P, true>(b, ntiles, smem, hi, ids, s);
	else launch_push_mix_pg<P, false>(b, ntiles, smem, hi, ids, s);
}

cudaError_t launch_push_mix(const PushArgs &a, int ntiles, size_t smem, int ppt, cudaStream_t s)
{
	if(!ppt_supported(ppt)) return cudaErrorInvalidValue;
	cudaError_t e = push_mix_attrs();
	if(e != cudaSuccess) return e;
	for(int sp = 0; sp < a.nspecies; sp++)
	{
		const PushArgs b = species_args(a, sp);
		const bool ids = b.mix[0].id != nullptr;
		const bool hi = push_mix_hi(smem, ids, ppt, b.g.pow2 != 0);
		if(ppt == 1) launch_push_mix_p<1>(b, ntiles, smem, hi, ids, s);
		else if(ppt == 4) launch_push_mix_p<4>(b, ntiles, smem, hi, ids, s);
		else launch_push_mix_p<2>(b, ntiles, smem, hi, ids, s);
	}
	return cudaSuccess;
}

void launch_spill_mix(const SpillArgs &a, cudaStream_t s)
{
	k_spill<Mix><<<152, kPushThreads, 0, s>>>(a);
}

cudaError_t launch_poisson_mix(const Grid &g, const long long *rho, double qinv, const long long *mean,
		float2 *spec, const float2 *twx, const float2 *twy, const double *cosx,
		const double *cosy, float *phi, cudaStream_t s, const float *Gt, double mean0)
{
	cudaError_t e = g_poisson_mix_once.run([] {
		return set_max_dyn_smem({(const void *) k_rows_fwd<float>, (const void *) k_cols<float>,
				(const void *) k_rows_inv<float>}, 200 * 1024);
	});
	if(e != cudaSuccess) return e;
	poisson_launch<float>(g, rho, qinv, mean, spec, twx, twy, cosx, cosy, phi, s, nullptr, 0.0, Gt,
			mean0);
	return cudaSuccess;
}

} // namespace cpic
