// cpic_fp64.cu -- FP64 ("plain") form of the step.  Compiled with
// --fmad=false so that every FP64 expression rounds exactly as the
// reference's C code does (no FMA contraction).
#include <algorithm>
#include "cpic_common.cuh"
#include "cpic_push.cuh"
#include "cpic_fft.cuh"

namespace cpic {

// field_E_compute, src/field.c:358-416: E = -grad(phi) by central
// differences, rows 0..ny (row ny is the south ghost), periodic through the
// phi ghosts (src/comm_field.c:140-201), which equals periodic indexing.
__global__ void k_E_f64(Grid g, const double *phi, double *Ex, double *Ey)
{
	double dx2 = 2 * g.dx, dy2 = 2 * g.dy;
	// rows 0..ny over blockIdx.y (row ny is the south ghost: row 0 again)
	for(int iy = blockIdx.y; iy <= g.ny; iy += gridDim.y)
	{
		int y0 = iy - 1 < 0 ? g.ny - 1 : iy - 1;
		int y1 = iy + 1 >= g.ny ? iy + 1 - g.ny : iy + 1;
		int yc = iy >= g.ny ? iy - g.ny : iy;
		for(int ix = blockIdx.x * blockDim.x + threadIdx.x; ix < g.nx;
				ix += gridDim.x * blockDim.x)
		{
			int x0 = ix == 0 ? g.nx - 1 : ix - 1;
			int x1 = ix + 1 == g.nx ? 0 : ix + 1;
			int64_t i = (int64_t) iy * g.nx + ix;
			Ey[i] = (phi[(int64_t) y0 * g.nx + ix] - phi[(int64_t) y1 * g.nx + ix]) / dy2;
			Ex[i] = (phi[(int64_t) yc * g.nx + x0] - phi[(int64_t) yc * g.nx + x1]) / dx2;
		}
	}
}

void launch_E_f64(const Grid &g, const double *phi, double *Ex, double *Ey, cudaStream_t s)
{
	dim3 grid((g.nx + 255) / 256, 1);
	grid.y = (unsigned) std::min(g.ny + 1, std::max(1, 4096 / (int) grid.x));
	k_E_f64<<<grid, 256, 0, s>>>(g, phi, Ex, Ey);
}

// E at every particle (interpolate_f2p_E), written by particle id.  One
// block per tile.
__global__ void k_gather_f64(Grid g, StoreF64 st, const int64_t *base, const int32_t *cnt,
		const double *Ex, const double *Ey, double *ex_out, double *ey_out)
{
	int t = blockIdx.x;
	int n = cnt[t];
	int64_t b = base[t];
	for(int i = threadIdx.x; i < n; i += blockDim.x)
	{
		double w[4];
		int i0x, i0y;
		double x = st.x[b + i], y = st.y[b + i];
		F64::weights(g, x, y, w, i0x, i0y);
		i0x = min(max(i0x, 0), g.nx);
		i0y = min(max(i0y, 0), g.ny);
		double ex, ey;
		F64::gather(Ex, Ey, g, w, i0x, i0y, ex, ey);
		int id = st.id[b + i];
		ex_out[id] = ex;
		ey_out[id] = ey;
	}
}

void launch_gather_f64_tiles(const Grid &g, const StoreF64 &st, const int64_t *base,
		const int32_t *cnt, int ntiles, const double *Ex, const double *Ey,
		double *ex_out, double *ey_out, cudaStream_t s)
{
	k_gather_f64<<<ntiles, 256, 0, s>>>(g, st, base, cnt, Ex, Ey, ex_out, ey_out);
}

static PerDeviceOnce g_push_f64_once, g_poisson_f64_once;

// The fused kernel's instance for P particles per thread.
static const void *push_f64_fn(int P)
{
	switch(P)
	{
		case 1: return (const void *) k_push<F64, F64::kMinBlocks, true, 1>;
		case 4: return (const void *) k_push<F64, F64::kMinBlocks, true, 4>;
		default: return (const void *) k_push<F64, F64::kMinBlocks, true, 2>;
	}
}

static cudaError_t push_f64_attrs()
{
	return g_push_f64_once.run([] {
		return set_max_dyn_smem({push_f64_fn(1), push_f64_fn(2), push_f64_fn(4)}, 200 * 1024, true);
	});
}

int push_f64_blocks_per_sm(size_t smem, int ppt)
{
	if(!ppt_supported(ppt) || push_f64_attrs() != cudaSuccess)
		return 0;
	int b = 0;
	if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, push_f64_fn(ppt), kPushThreads, smem)
			!= cudaSuccess)
		return 0;
	return b;
}

cudaError_t launch_push_f64(const PushArgs &a, int ntiles, size_t smem, int ppt, cudaStream_t s)
{
	if(!ppt_supported(ppt)) return cudaErrorInvalidValue;
	cudaError_t e = push_f64_attrs();
	if(e != cudaSuccess) return e;
	for(int sp = 0; sp < a.nspecies; sp++)
	{
		const PushArgs b = species_args(a, sp);
		if(ppt == 1) k_push<F64, F64::kMinBlocks, true, 1><<<ntiles, kPushThreads, smem, s>>>(b);
		else if(ppt == 4) k_push<F64, F64::kMinBlocks, true, 4><<<ntiles, kPushThreads, smem, s>>>(b);
		else k_push<F64, F64::kMinBlocks, true, 2><<<ntiles, kPushThreads, smem, s>>>(b);
	}
	return cudaSuccess;
}

void launch_spill_f64(const SpillArgs &a, cudaStream_t s)
{
	k_spill<F64><<<152, kPushThreads, 0, s>>>(a);
}

cudaError_t launch_poisson_f64(const Grid &g, const long long *rho, double qinv,
		double2 *spec, const double2 *twx, const double2 *twy, const double *cosx,
		const double *cosy, double *phi, cudaStream_t s, const long long *rho_lo, double qinv_lo,
		const double *Gt)
{
	cudaError_t e = g_poisson_f64_once.run([] {
		return set_max_dyn_smem({(const void *) k_rows_fwd<double>, (const void *) k_cols<double>,
				(const void *) k_rows_inv<double>}, 200 * 1024);
	});
	if(e != cudaSuccess) return e;
	poisson_launch<double>(g, rho, qinv, nullptr, spec, twx, twy, cosx, cosy, phi, s, rho_lo, qinv_lo,
			Gt);
	return cudaSuccess;
}

} // namespace cpic
