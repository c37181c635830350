// cpic_peak.cu -- FP64 arithmetic peak of the current GPU, the denominator of
// the FP64 plain form's roofline.  No counterpart in the reference.
//
// Every thread runs kChains independent chains of dependent FP64
// fused multiply-adds (x = x * a + b with |a| < 1, so the values stay
// bounded and never become subnormal); enough resident warps hide the FMA
// latency, so the launch runs at the FP64 pipes' issue rate.  FLOPs = 2 per
// FMA.  Changes no device setting.
#include <cstdio>

#include "../../include/cpic_gpu.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_fp64_fma(int64_t iters, double a, double b, double *sink)
{
	double x[kChains];
	#pragma unroll
	for(int c = 0; c < kChains; c++)
		x[c] = (double) (threadIdx.x + c) * 1e-3;
	for(int64_t i = 0; i < iters; i++)
	{
		#pragma unroll
		for(int c = 0; c < kChains; c++)
			x[c] = fma(x[c], a, b);
	}
	double s = 0.0;
	#pragma unroll
	for(int c = 0; c < kChains; c++)
		s += x[c];
	// one store per thread keeps the chains alive; a value that cannot occur
	// (the chains converge to b / (1 - a) > 0) guards it
	if(s == -1.0)
		sink[threadIdx.x] = s;
}

} // namespace

extern "C" CPIC_API int
cpic_fp64_peak(int64_t iters, double *gflops, double *ms)
{
	if(iters <= 0 || !gflops) return CPIC_EINVAL;
	int dev = 0, sms = 0, per_sm = 0;
	if(cudaGetDevice(&dev) != cudaSuccess) return CPIC_ENODEV;
	if(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
		return CPIC_ECUDA;
	if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fp64_fma, kThreads, 0) != cudaSuccess)
		return CPIC_ECUDA;
	const int blocks = sms * (per_sm > 0 ? per_sm : 1);
	double *sink = nullptr;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	int r = CPIC_OK;
	float t = 0.0f;
	if(cudaMalloc((void **) &sink, kThreads * sizeof(double)) != cudaSuccess) return CPIC_ENOMEM;
	if(cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
		r = CPIC_ECUDA;
	if(r == CPIC_OK)
	{
		// warm-up launch (clocks up, code loaded), then the timed one
		k_fp64_fma<<<blocks, kThreads>>>(iters / 8 + 1, 0.999999, 1e-6, sink);
		cudaEventRecord(e0);
		k_fp64_fma<<<blocks, kThreads>>>(iters, 0.999999, 1e-6, sink);
		cudaEventRecord(e1);
		if(cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess
				|| cudaEventElapsedTime(&t, e0, e1) != cudaSuccess)
			r = CPIC_ECUDA;
	}
	if(e0) cudaEventDestroy(e0);
	if(e1) cudaEventDestroy(e1);
	cudaFree(sink);
	if(r != CPIC_OK) return r;
	double flops = 2.0 * kChains * (double) iters * (double) blocks * kThreads;
	*gflops = flops / (t * 1e-3) / 1e9;
	if(ms) *ms = t;
	return CPIC_OK;
}
