// cpic_fft.cuh -- periodic FFT Poisson solver for any grid (radix-4/2
// passes for power-of-two sides, mixed-radix passes otherwise), templated
// on the real type (double for the FP64 form, float for the mixed form).
//
// Replaces MFT_solve (src/solver.c:465-509): phi = IFFT(G * FFT(rho)) / (nx
// ny) with G(kx,ky) = 1 / (2 (cos(2 pi kx/nx) + cos(2 pi ky/ny)) - 4) and
// G(0,0) = 0 (solver.c:269-280).  Three kernels, all working in shared
// memory with Stockham passes (self-sorting, no bit reversal):
//   rows_fwd : two real rows packed as one complex row, FFT along x, split
//              into the two half spectra (nx/2+1 bins each; the last row
//              of an odd ny alone);
//   cols     : a block of spectrum columns, FFT along y, multiply by G,
//              inverse FFT along y (the Green's function never leaves
//              shared memory);
//   rows_inv : two half spectra packed into one Hermitian-extended row,
//              inverse FFT, real and imaginary parts are the two phi rows,
//              divided by nx*ny as MFT_normalize does (solver.c:366).
#pragma once
#include <cuda_runtime.h>
#include "cpic_common.cuh"

namespace cpic {

template <typename T> struct Cx;
template <> struct Cx<double> { typedef double2 t; };
template <> struct Cx<float> { typedef float2 t; };

template <typename C>
__device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C>
__device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C>
__device__ __forceinline__ C cmul(C a, C b)
{
	C r;
	r.x = a.x * b.x - a.y * b.y;
	r.y = a.x * b.y + a.y * b.x;
	return r;
}

// Twiddle exp(-2 pi i m / n) for 0 <= m < n from the half table
// tw[m] (m < n/2): exp(-2 pi i (m + n/2) / n) = -exp(-2 pi i m / n).
template <typename C>
__device__ __forceinline__ C twiddle(const C *tw, int m, int half, int sign)
{
	C w = m < half ? tw[m] : tw[m - half];
	if(m >= half) { w.x = -w.x; w.y = -w.y; }
	if(sign > 0) w.y = -w.y;
	return w;
}

// nb independent length-n sequences stored back to back in `a`; `b` is
// scratch of the same size.  tw[k] = exp(-2 pi i k / n), k < n/2.  sign
// -1 forward, +1 inverse (unnormalised).  Returns the buffer holding the
// result.  Must be called by the whole block.
//
// Stockham autosort passes (no bit reversal): one radix-2 pass first when
// log2 n is odd (sub-transforms of length 1: unit twiddles), then radix-4
// passes.  A radix-4 pass with sub-transform length Ns takes x[j + q n/4],
// q = 0..3, twiddles them by exp(sign 2 pi i q k / (4 Ns)) (k = j mod Ns)
// and writes their 4-point DFT to y[4 (j - k) + k + p Ns], p = 0..3: half
// as many passes and block barriers as radix 2.
template <typename C>
__device__ C *fft_smem(C *a, C *b, int n, int log2n, int nb, int sign, const C *tw)
{
	const int half = n >> 1;
	int Ns = 1, s = 0;
	if(log2n & 1)
	{
		const int total = half * nb;
		for(int idx = threadIdx.x; idx < total; idx += blockDim.x)
		{
			int seq = idx >> (log2n - 1);
			int j = idx & (half - 1);
			const C *x = a + seq * n;
			C *y = b + seq * n;
			C a0 = x[j], a1 = x[j + half];
			y[2 * j] = cadd(a0, a1);
			y[2 * j + 1] = csub(a0, a1);
		}
		__syncthreads();
		C *t = a; a = b; b = t;
		Ns = 2;
		s = 1;
	}
	const int q4 = n >> 2;
	for(; Ns < n; Ns <<= 2, s += 2)
	{
		const int total = q4 * nb;
		const int sh = log2n - 2 - s;        // n / (4 Ns) = 2^sh
		for(int idx = threadIdx.x; idx < total; idx += blockDim.x)
		{
			int seq = idx >> (log2n - 2);
			int j = idx & (q4 - 1);
			const C *x = a + seq * n;
			C *y = b + seq * n;
			int k = j & (Ns - 1);
			C v0 = x[j];
			C v1 = cmul(x[j + q4], twiddle(tw, k << sh, half, sign));
			C v2 = cmul(x[j + 2 * q4], twiddle(tw, (2 * k) << sh, half, sign));
			C v3 = cmul(x[j + 3 * q4], twiddle(tw, (3 * k) << sh, half, sign));
			C t0 = cadd(v0, v2), t1 = csub(v0, v2), t2 = cadd(v1, v3), t3 = csub(v1, v3);
			// t3 times -i (forward) or +i (inverse)
			C r3;
			if(sign < 0) { r3.x = t3.y; r3.y = -t3.x; }
			else { r3.x = -t3.y; r3.y = t3.x; }
			int o = ((j - k) << 2) + k;
			y[o] = cadd(t0, t2);
			y[o + Ns] = cadd(t1, r3);
			y[o + 2 * Ns] = csub(t0, t2);
			y[o + 3 * Ns] = csub(t1, r3);
		}
		__syncthreads();
		C *t = a; a = b; b = t;
	}
	return a;
}

// Any n >= 2 (the power-of-two passes above when n is one): mixed-radix
// Stockham passes over the prime factors of n (4s first, then 2, then the
// odd primes in increasing order), each pass computing every output
// directly from its r inputs.  A pass of radix r after sub-transforms of
// length Ns (the product of the radices before it) writes
//   y[(j - k) r + k + p Ns] = sum_q x[j + q n/r] exp(sign 2 pi i q (k + p Ns) / (r Ns))
// for j < n/r, k = j mod Ns, p < r: the twiddle and the r-point DFT in
// one exponent, read from the full table tw[m] = exp(-2 pi i m / n), m < n
// (conjugated for the inverse).  O(n r) work per pass: a length with a
// large prime factor transforms correctly but slowly.
template <typename C>
__device__ C *fft_smem_any(C *a, C *b, int n, int nb, int sign, const C *tw)
{
	int rem = n, Ns = 1;
	while(rem > 1)
	{
		int r;
		if(rem % 4 == 0) r = 4;
		else if(rem % 2 == 0) r = 2;
		else
		{
			r = 3;
			while(rem % r) r += 2;
		}
		const int m = n / r;                 // outputs per output digit p
		const int step0 = n / (r * Ns);      // table stride of one unit of k + p Ns
		const int total = n * nb;
		for(int idx = threadIdx.x; idx < total; idx += blockDim.x)
		{
			const int seq = idx / n, o = idx - seq * n;
			const int p = o / m, j = o - p * m;
			const int k = j % Ns;
			const C *x = a + (size_t) seq * n;
			const int step = (k + p * Ns) * step0;   // < n
			C acc = x[j];
			int t = 0;
			for(int q = 1; q < r; q++)
			{
				t += step;
				if(t >= n) t -= n;
				C w = tw[t];
				if(sign > 0) w.y = -w.y;
				acc = cadd(acc, cmul(x[j + q * m], w));
			}
			b[(size_t) seq * n + (j - k) * r + k + p * Ns] = acc;
		}
		__syncthreads();
		C *t = a; a = b; b = t;
		Ns *= r;
		rem /= r;
	}
	return a;
}

// The transform of fft_smem for a power-of-two n (log2n its exponent), of
// fft_smem_any otherwise.
template <typename C>
__device__ __forceinline__ C *fft_any(C *a, C *b, int n, int log2n, int nb, int sign, const C *tw)
{
	if((1 << log2n) == n)
		return fft_smem<C>(a, b, n, log2n, nb, sign, tw);
	return fft_smem_any<C>(a, b, n, nb, sign, tw);
}

// The kernels below are static: the FP64 units (built without FMA
// contraction) and the mixed and adjoint units (built with it) each get their
// own copy, so a launch always runs the device code of the unit that makes
// it, and a kernel attribute set in one unit leaves the other units' kernels
// alone.

// rho (fixed point, ny x nx) -> spec (ny x (nx/2+1)).  One block per row
// pair.  value = (double) acc * qinv - mean, where the mean (the k = 0
// mode, removed in FP64 before the FP32 transform of the mixed form, so
// that the transform's rounding scales with the fluctuations, not with the
// total charge) comes from the exact integer sum rsum, or is mean0 when
// rsum is null.  G(0,0) = 0 discards whatever is left of the mode, so mean0
// may be the charge the particles carry (the deposit's weight rounding
// leaves a residue of ~2^-17 of it).  FP64 form: no removal (as the
// reference).
// rho_lo (FP64 form, may be null): the remainder word at scale qinv_lo.
template <typename T>
static __global__ void k_rows_fwd(int nx, int log2nx, int ny, const long long *rho, double qinv,
		const long long *rsum, typename Cx<T>::t *spec, const typename Cx<T>::t *tw,
		const long long *rho_lo, double qinv_lo, double mean0)
{
	typedef typename Cx<T>::t C;
	extern __shared__ unsigned char smem_raw[];
	C *a = reinterpret_cast<C *>(smem_raw);
	C *b = a + nx;
	int r0 = 2 * blockIdx.x;
	const bool two = r0 + 1 < ny;            // an odd ny leaves the last row alone
	int nh = nx / 2 + 1;
	double m = rsum ? (double) *rsum * qinv / ((double) nx * (double) ny) : mean0;
	for(int i = threadIdx.x; i < nx; i += blockDim.x)
	{
		int64_t ia = (int64_t) r0 * nx + i, ib = (int64_t) (r0 + 1) * nx + i;
		double va = (double) rho[ia] * qinv - m;
		double vb = two ? (double) rho[ib] * qinv - m : 0.0;
		if(rho_lo)
		{
			va += (double) rho_lo[ia] * qinv_lo;
			if(two) vb += (double) rho_lo[ib] * qinv_lo;
		}
		C z; z.x = (T) va; z.y = (T) vb;
		a[i] = z;
	}
	__syncthreads();
	C *Z = fft_any<C>(a, b, nx, log2nx, 1, -1, tw);
	for(int k = threadIdx.x; k < nh; k += blockDim.x)
	{
		C p = Z[k];
		C q = Z[k == 0 ? 0 : nx - k];
		q.y = -q.y;                          // conj(Z[-k])
		C A, B;
		A.x = (p.x + q.x) * (T) 0.5;
		A.y = (p.y + q.y) * (T) 0.5;
		// (p - q) / (2i) = -i (p - q) / 2
		B.x = (p.y - q.y) * (T) 0.5;
		B.y = -(p.x - q.x) * (T) 0.5;
		spec[(int64_t) r0 * nh + k] = A;
		if(two) spec[(int64_t) (r0 + 1) * nh + k] = B;
	}
}

// The Green's function G(kx, ky) = 1 / (2 (cos(2 pi kx/nx) + cos(2 pi
// ky/ny)) - 4), G(0, 0) = 0 (solver.c:269-280), stored once per context in
// column order Gt[kx * ny + ky] (the order k_cols reads it), as type T.
// Evaluated in FP64 from the same cosine tables and with the same
// operations as k_cols's fallback below, so both give identical values.
template <typename T>
static __global__ void k_green(int nx, int ny, const double *cosx, const double *cosy, T *Gt)
{
	int nh = nx / 2 + 1;
	int64_t total = (int64_t) nh * ny;
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < total;
			i += (int64_t) gridDim.x * blockDim.x)
	{
		int kx = (int) (i / ny), row = (int) (i - (int64_t) kx * ny);
		double G = (kx == 0 && row == 0) ? 0.0 : 1.0 / (2.0 * (cosx[kx] + cosy[row]) - 4.0);
		Gt[i] = (T) G;
	}
}

// Columns [c0, c0 + cb) of spec: FFT along y, multiply by G, inverse FFT.
// Gt: the precomputed Green's function (k_green), or null to evaluate it
// from the cosine tables (FP64 division per element: slow on a GPU with
// few FP64 units, kept for callers without the table).
template <typename T>
static __global__ void k_cols(int nx, int ny, int log2ny, int cb, typename Cx<T>::t *spec,
		const typename Cx<T>::t *tw, const double *cosx, const double *cosy, const T *Gt)
{
	typedef typename Cx<T>::t C;
	extern __shared__ unsigned char smem_raw[];
	int nh = nx / 2 + 1;
	int c0 = blockIdx.x * cb;
	int ncol = min(cb, nh - c0);
	C *a = reinterpret_cast<C *>(smem_raw);
	C *b = a + (size_t) cb * ny;
	// element idx of the block's columns: row idx / ncol, column idx % ncol
	// (a shift and a mask when ncol is a power of two, as it is except
	// for small grids)
	const int lg = (ncol & (ncol - 1)) == 0 ? __ffs(ncol) - 1 : -1;
	for(int idx = threadIdx.x; idx < ncol * ny; idx += blockDim.x)
	{
		int row = lg >= 0 ? idx >> lg : idx / ncol, c = idx - row * ncol;
		a[c * ny + row] = spec[(int64_t) row * nh + c0 + c];
	}
	__syncthreads();
	C *X = fft_any<C>(a, b, ny, log2ny, ncol, -1, tw);
	if(Gt)
	{
		const T *Gc = Gt + (size_t) c0 * ny;    // columns are contiguous
		for(int idx = threadIdx.x; idx < ncol * ny; idx += blockDim.x)
		{
			T G = Gc[idx];
			C v = X[idx];
			v.x = v.x * G;
			v.y = v.y * G;
			X[idx] = v;
		}
	}
	else
	{
		for(int idx = threadIdx.x; idx < ncol * ny; idx += blockDim.x)
		{
			int c = idx / ny, row = idx - c * ny;
			int kx = c0 + c;
			double G = (kx == 0 && row == 0) ? 0.0 : 1.0 / (2.0 * (cosx[kx] + cosy[row]) - 4.0);
			C v = X[idx];
			v.x = v.x * (T) G;
			v.y = v.y * (T) G;
			X[idx] = v;
		}
	}
	__syncthreads();
	C *Y = (X == a) ? b : a;
	C *R = fft_any<C>(X, Y, ny, log2ny, ncol, +1, tw);
	for(int idx = threadIdx.x; idx < ncol * ny; idx += blockDim.x)
	{
		int row = lg >= 0 ? idx >> lg : idx / ncol, c = idx - row * ncol;
		spec[(int64_t) row * nh + c0 + c] = R[c * ny + row];
	}
}

// spec -> phi (ny x nx real).  One block per row pair.
template <typename T>
static __global__ void k_rows_inv(int nx, int log2nx, int ny, const typename Cx<T>::t *spec,
		const typename Cx<T>::t *tw, T *phi)
{
	typedef typename Cx<T>::t C;
	extern __shared__ unsigned char smem_raw[];
	C *a = reinterpret_cast<C *>(smem_raw);
	C *b = a + nx;
	int r0 = 2 * blockIdx.x;
	const bool two = r0 + 1 < ny;            // an odd ny leaves the last row alone
	int nh = nx / 2 + 1;
	for(int k = threadIdx.x; k < nh; k += blockDim.x)
	{
		C A = spec[(int64_t) r0 * nh + k];
		C B;
		if(two) B = spec[(int64_t) (r0 + 1) * nh + k];
		else { B.x = (T) 0; B.y = (T) 0; }
		if(k == 0 || 2 * k == nx)
		{
			// c2r uses only the real part of the DC and Nyquist bins
			C y; y.x = A.x; y.y = B.x;
			a[k] = y;
		}
		else
		{
			C y;
			y.x = A.x - B.y; y.y = A.y + B.x;     // A + iB
			a[k] = y;
			y.x = A.x + B.y; y.y = B.x - A.y;     // conj(A) + i conj(B)
			a[nx - k] = y;
		}
	}
	__syncthreads();
	C *Y = fft_any<C>(a, b, nx, log2nx, 1, +1, tw);
	T N = (T) ((double) nx * (double) ny);
	for(int i = threadIdx.x; i < nx; i += blockDim.x)
	{
		C v = Y[i];
		phi[(int64_t) r0 * nx + i] = v.x / N;
		if(two) phi[(int64_t) (r0 + 1) * nx + i] = v.y / N;
	}
}

// Real-valued input (ny x nx of T) -> spec, otherwise as k_rows_fwd.  Used
// by the adjoint, whose source term (rho-bar) is not a charge sum.
template <typename T>
static __global__ void k_rows_fwd_real(int nx, int log2nx, int ny, const T *in,
		typename Cx<T>::t *spec, const typename Cx<T>::t *tw)
{
	typedef typename Cx<T>::t C;
	extern __shared__ unsigned char smem_raw[];
	C *a = reinterpret_cast<C *>(smem_raw);
	C *b = a + nx;
	int r0 = 2 * blockIdx.x;
	const bool two = r0 + 1 < ny;
	int nh = nx / 2 + 1;
	for(int i = threadIdx.x; i < nx; i += blockDim.x)
	{
		C z;
		z.x = in[(int64_t) r0 * nx + i];
		z.y = two ? in[(int64_t) (r0 + 1) * nx + i] : (T) 0;
		a[i] = z;
	}
	__syncthreads();
	C *Z = fft_any<C>(a, b, nx, log2nx, 1, -1, tw);
	for(int k = threadIdx.x; k < nh; k += blockDim.x)
	{
		C p = Z[k];
		C q = Z[k == 0 ? 0 : nx - k];
		q.y = -q.y;
		C A, B;
		A.x = (p.x + q.x) * (T) 0.5;
		A.y = (p.y + q.y) * (T) 0.5;
		B.x = (p.y - q.y) * (T) 0.5;
		B.y = -(p.x - q.x) * (T) 0.5;
		spec[(int64_t) r0 * nh + k] = A;
		if(two) spec[(int64_t) (r0 + 1) * nh + k] = B;
	}
}

template <typename T>
static void poisson_launch(const Grid &g, const long long *rho, double qinv, const long long *mean,
		typename Cx<T>::t *spec, const typename Cx<T>::t *twx, const typename Cx<T>::t *twy,
		const double *cosx, const double *cosy, T *phi, cudaStream_t s,
		const long long *rho_lo = nullptr, double qinv_lo = 0.0, const T *Gt = nullptr,
		double mean0 = 0.0)
{
	typedef typename Cx<T>::t C;
	int log2nx = 0, log2ny = 0;
	while((1 << log2nx) < g.nx) log2nx++;
	while((1 << log2ny) < g.ny) log2ny++;
	int rthreads = g.nx / 2 < 512 ? (g.nx / 2 < 32 ? 32 : g.nx / 2) : 512;
	size_t rsm = 2 * (size_t) g.nx * sizeof(C);
	k_rows_fwd<T><<<(g.ny + 1) / 2, rthreads, rsm, s>>>(g.nx, log2nx, g.ny, rho, qinv, mean, spec, twx,
			rho_lo, qinv_lo, mean0);
	int nh = g.nx / 2 + 1;
	// columns per block: up to 64 KB of shared memory (two buffers), so
	// that several blocks share an SM
	int cb = (int) ((64 * 1024) / (2 * (size_t) g.ny * sizeof(C)));
	if(cb < 1) cb = 1;
	if(cb > nh) cb = nh;
	size_t csm = 2 * (size_t) cb * g.ny * sizeof(C);
	int cthreads = 512;
	k_cols<T><<<(nh + cb - 1) / cb, cthreads, csm, s>>>(g.nx, g.ny, log2ny, cb, spec, twy, cosx, cosy,
			Gt);
	k_rows_inv<T><<<(g.ny + 1) / 2, rthreads, rsm, s>>>(g.nx, log2nx, g.ny, spec, twx, phi);
}

// out = IFFT(G FFT(in)) / (nx ny) for a real ny x nx input: the same linear
// operator as poisson_launch (symmetric, so it is also its own adjoint).
template <typename T>
static void poisson_launch_real(const Grid &g, const T *in, typename Cx<T>::t *spec,
		const typename Cx<T>::t *twx, const typename Cx<T>::t *twy, const double *cosx,
		const double *cosy, T *out, cudaStream_t s)
{
	typedef typename Cx<T>::t C;
	int log2nx = 0, log2ny = 0;
	while((1 << log2nx) < g.nx) log2nx++;
	while((1 << log2ny) < g.ny) log2ny++;
	int rthreads = g.nx / 2 < 512 ? (g.nx / 2 < 32 ? 32 : g.nx / 2) : 512;
	size_t rsm = 2 * (size_t) g.nx * sizeof(C);
	k_rows_fwd_real<T><<<(g.ny + 1) / 2, rthreads, rsm, s>>>(g.nx, log2nx, g.ny, in, spec, twx);
	int nh = g.nx / 2 + 1;
	int cb = (int) ((64 * 1024) / (2 * (size_t) g.ny * sizeof(C)));
	if(cb < 1) cb = 1;
	if(cb > nh) cb = nh;
	size_t csm = 2 * (size_t) cb * g.ny * sizeof(C);
	k_cols<T><<<(nh + cb - 1) / cb, 512, csm, s>>>(g.nx, g.ny, log2ny, cb, spec, twy, cosx, cosy,
			nullptr);
	k_rows_inv<T><<<(g.ny + 1) / 2, rthreads, rsm, s>>>(g.nx, log2nx, g.ny, spec, twx, out);
}

} // namespace cpic
