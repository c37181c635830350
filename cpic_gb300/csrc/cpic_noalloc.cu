// cpic_noalloc.cu -- an FP64 periodic Poisson solve that allocates nothing.
//
// Some callers cannot allocate device memory: applications that have
// reserved the whole device up front for their own pool or run under a fixed
// memory budget, and latency-critical host threads on which cudaMalloc or
// cudaFree (which may synchronise the device) must not appear.  For them,
// cpic_poisson_noalloc solves the same periodic Poisson problem as the
// context's field stage (the MFT solve of the reference, solver.c:465-509)
// with every piece of scratch -- the half spectrum, the FFT twiddles and the
// Green's-function cosines -- in one file-scope __device__ array of fixed
// size.  The caller passes its own input and output device buffers.
//
// The array is held by every GPU that loads this library until the process
// exits (about 2.1 MB).  In host code the symbol is only a host-side
// stand-in, never a device address: its device address is obtained once per
// device with cudaGetSymbolAddress, on the first call made with that device
// current, and passed to the kernels.  All calls share the array and it keeps
// the last call's contents; each call rewrites everything it reads before
// reading it, so nothing carries over.  Calls that overlap on the GPU (for
// example from two streams at once) race on the array and must be
// serialised by the caller.
#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/cpic_gpu.h"
#include "cpic_common.cuh"
#include "cpic_fft.cuh"

namespace {

using namespace cpic;

constexpr int kMaxN = CPIC_NOALLOC_MAX_N;            // nx, ny <= kMaxN
constexpr size_t kSpecElems = (size_t) kMaxN * (kMaxN / 2 + 1);
// layout: [spectrum kSpecElems double2][twx kMaxN/2 double2][twy kMaxN/2 double2]
//         [cosx kMaxN double][cosy kMaxN double]
constexpr size_t kScratchBytes = kSpecElems * sizeof(double2) + 2 * (kMaxN / 2) * sizeof(double2)
	+ 2 * (size_t) kMaxN * sizeof(double);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
static void *g_scratch_addr[kMaxDevices];
static std::mutex g_setup_lock;

// Twiddles exp(-2 pi i k / n) and cosines cos(2 pi j / n), computed on the
// device (sincospi: correctly scaled, ~1 ulp).
__global__ void k_noalloc_tables(int nx, int ny, double2 *twx, double2 *twy, double *cosx,
		double *cosy)
{
	for(int k = blockIdx.x * blockDim.x + threadIdx.x; k < kMaxN; k += gridDim.x * blockDim.x)
	{
		double s, c;
		if(k < nx / 2) { sincospi(-2.0 * k / nx, &s, &c); twx[k] = make_double2(c, s); }
		if(k < ny / 2) { sincospi(-2.0 * k / ny, &s, &c); twy[k] = make_double2(c, s); }
		if(k < nx) cosx[k] = cospi(2.0 * k / nx);
		if(k < ny) cosy[k] = cospi(2.0 * k / ny);
	}
}

// rho (FP64, ny x nx) -> half spectra, two rows per block (the context's
// rows_fwd reads fixed-point charge; this one reads the caller's doubles).
__global__ void k_noalloc_rows_fwd(int nx, int log2nx, const double *rho, double2 *spec,
		const double2 *tw)
{
	extern __shared__ unsigned char smem_raw[];
	double2 *a = reinterpret_cast<double2 *>(smem_raw);
	double2 *b = a + nx;
	int r0 = 2 * blockIdx.x;
	int nh = nx / 2 + 1;
	for(int i = threadIdx.x; i < nx; i += blockDim.x)
		a[i] = make_double2(rho[(int64_t) r0 * nx + i], rho[(int64_t) (r0 + 1) * nx + i]);
	__syncthreads();
	double2 *Z = fft_smem<double2>(a, b, nx, log2nx, 1, -1, tw);
	for(int k = threadIdx.x; k < nh; k += blockDim.x)
	{
		double2 p = Z[k], q = Z[(nx - k) & (nx - 1)];
		q.y = -q.y;
		spec[(int64_t) r0 * nh + k] = make_double2((p.x + q.x) * 0.5, (p.y + q.y) * 0.5);
		spec[(int64_t) (r0 + 1) * nh + k] = make_double2((p.y - q.y) * 0.5, -(p.x - q.x) * 0.5);
	}
}

// Device address of the scratch array for the current device, looked up
// once per device, together with the kernels' shared-memory limits (a
// kernel attribute belongs to the device it was set on).  A device is marked
// ready only when every step succeeded, so a failed set-up is retried by the
// next call.
static int scratch_for_current_device(void **out)
{
	int dev = -1;
	if(cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
		return CPIC_ENODEV;
	std::lock_guard<std::mutex> lk(g_setup_lock);
	if(!g_scratch_addr[dev])
	{
		void *p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if(e == cudaSuccess && !p)
			e = cudaErrorInvalidSymbol;
		// the largest blocks: two rows of kMaxN complex values, and the
		// columns' two buffers of at most 128 KB together
		if(e == cudaSuccess)
			e = set_max_dyn_smem({(const void *) k_noalloc_rows_fwd,
					(const void *) k_rows_inv<double>}, 2 * kMaxN * (int) sizeof(double2));
		if(e == cudaSuccess)
			e = set_max_dyn_smem({(const void *) k_cols<double>}, 128 * 1024);
		if(e != cudaSuccess)
		{
			fprintf(stderr, "cpic_poisson_noalloc: set-up on device %d failed: %s\n", dev,
					cudaGetErrorString(e));
			return CPIC_ECUDA;
		}
		g_scratch_addr[dev] = p;
	}
	*out = g_scratch_addr[dev];
	return CPIC_OK;
}

// One launch with its own error code (cudaLaunchKernel reports this launch's
// configuration error, not an earlier one left pending on the thread).
template <class T> struct same { typedef T type; };

template <typename... A>
static cudaError_t launch(void (*k)(A...), int blocks, int threads, size_t smem, cudaStream_t s,
		typename same<A>::type... args)
{
	void *argv[] = {(void *) &args...};
	return cudaLaunchKernel((const void *) k, dim3(blocks), dim3(threads), argv, smem, s);
}

} // namespace

extern "C" CPIC_API int
cpic_poisson_noalloc(const double *rho, double *phi, int64_t nx, int64_t ny, void *stream)
{
	if(!rho || !phi) return CPIC_EINVAL;
	if(nx < 4 || ny < 4 || (nx & (nx - 1)) || (ny & (ny - 1)))
		return CPIC_EINVAL;
	if(nx > kMaxN || ny > kMaxN)
	{
		fprintf(stderr, "cpic_poisson_noalloc: grid %lldx%lld exceeds the %dx%d maximum of the "
				"built-in scratch array\n", (long long) nx, (long long) ny, kMaxN, kMaxN);
		return CPIC_EINVAL;
	}
	void *base = nullptr;
	int r = scratch_for_current_device(&base);
	if(r) return r;
	cudaStream_t s = (cudaStream_t) stream;
	unsigned char *p = (unsigned char *) base;
	double2 *spec = (double2 *) p;
	double2 *twx = (double2 *) (p + kSpecElems * sizeof(double2));
	double2 *twy = twx + kMaxN / 2;
	double *cosx = (double *) (twy + kMaxN / 2);
	double *cosy = cosx + kMaxN;
	int nxi = (int) nx, nyi = (int) ny;
	int log2nx = 0, log2ny = 0;
	while((1 << log2nx) < nxi) log2nx++;
	while((1 << log2ny) < nyi) log2ny++;

	int rthreads = nxi / 2 < 32 ? 32 : (nxi / 2 > 512 ? 512 : nxi / 2);
	int nh = nxi / 2 + 1;
	int cb = (int) ((128 * 1024) / (2 * (size_t) nyi * sizeof(double2)));
	if(cb < 1) cb = 1;
	if(cb > nh) cb = nh;
	const size_t rsm = 2 * (size_t) nxi * sizeof(double2);
	const size_t csm = 2 * (size_t) cb * nyi * sizeof(double2);
	cudaError_t e = launch(k_noalloc_tables, (kMaxN + 255) / 256, 256, 0, s, nxi, nyi, twx, twy,
			cosx, cosy);
	if(e == cudaSuccess)
		e = launch(k_noalloc_rows_fwd, nyi / 2, rthreads, rsm, s, nxi, log2nx, rho, spec, twx);
	if(e == cudaSuccess)
		e = launch(k_cols<double>, (nh + cb - 1) / cb, 512, csm, s, nxi, nyi, log2ny, cb, spec, twy,
				cosx, cosy, nullptr);
	if(e == cudaSuccess)
		e = launch(k_rows_inv<double>, nyi / 2, rthreads, rsm, s, nxi, log2nx, nyi, spec, twx, phi);
	if(e != cudaSuccess)
	{
		fprintf(stderr, "cpic_poisson_noalloc: launch failed: %s\n", cudaGetErrorString(e));
		return CPIC_ECUDA;
	}
	return CPIC_OK;
}
