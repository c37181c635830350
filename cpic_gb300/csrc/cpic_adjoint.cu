// cpic_adjoint.cu -- differentiable run of the step and its hand-written
// adjoint: d(final field energy) / d(initial positions and velocities).
//
// Forward step j (j = 0 .. nsteps-1), the reference's order (sim.c:481-581):
//   rho_j = D(p_j)                 CIC deposit, -q/e0 per unit weight
//                                  (interpolate.c:282-346)
//   E_j   = -grad_h P rho_j        periodic FFT Poisson (solver.c:465-509)
//                                  and central differences (field.c:358-416)
//   e_i   = I(p_i; E_j)            CIC gather (interpolate.c:349-404)
//   u    <- M (u + h e) + h e      Boris for B along z, h = q dt'/(2m),
//                                  dt' = -dt/2 at j = 0 (mover.c:15-226)
//   p    <- wrap(p + dt u)         no move at j = 0 (mover.c:204-213)
// Loss: L = 1/2 e0 dx dy sum |E(D(p_N))|^2.
//
// Reverse step j, given the adjoints pb = dL/dp_{j+1} (without the deposit
// term of step j+1) and ub = dL/du_{j+1}:
//   pb   += c grad D(p_{j+1})^T rhob_{j+1}     (deposit adjoint = gather of
//                                                the weight gradients)
//   ut    = ub + move dt pb
//   vb    = M^T ut ;  eb = h (ut + vb) ;  ub = vb
//   pb   += grad I(p_j; E_j)^T eb              (gather's position term)
//   Eb_j  = sum_i w(p_j) eb_i                  (gather adjoint = deposit)
//   rhob_j = P^T (-grad_h)^T Eb_j = P div_h Eb_j
// and finally pb_0 += c grad D(p_0)^T rhob_0.  Only positions p_j and the
// grids E_j of a segment are needed in reverse (the kick is linear in u),
// so a segment of K steps is recomputed from its checkpoint (p, u) storing
// p_j and E_j, then swept backwards.
//
// Sums over particles into grids are 64-bit fixed point (integer atomics,
// order independent, deterministic).  The adjoint deposit's scale comes
// from a bound on |eb| computed on the device from the previous step's
// maxima, so it can never wrap.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/cpic_gpu.h"
#include "cpic_common.cuh"
#include "cpic_fft.cuh"

namespace cpic {
namespace adj {

struct AGrid {
	int nx, ny;
	double dx, dy, idx, idy, Lx, Ly;
};

// Boris kick of one iteration: u' = M (u + h e) + h e, M = [[a, s], [-s, a]]
// with t = Bz h, s = 2t / (1 + t^2), a = 1 - s t.
struct Kick {
	double h, t, s, a;
	int move;
};

struct Scale {
	double emul, einv;           // adjoint deposit fixed-point scale
	unsigned long long umax, pmax, rmax;  // |.| maxima as double bit patterns:
	                             // inputs of the next reverse step
	unsigned long long umax_n, pmax_n;    // written by the reverse step
};

template <typename T> struct V2T;
template <> struct V2T<double> { typedef double2 t; };
template <> struct V2T<float> { typedef float2 t; };

// CIC cell and fractions of a position in [0, L]; x == L maps to node 0.
template <typename T>
__device__ __forceinline__ void cell(const AGrid &g, T x, T y, int &ix, int &iy, int &ix1, int &iy1,
		T &fx, T &fy)
{
	T gx = x * (T) g.idx, gy = y * (T) g.idy;
	T flx = floor(gx), fly = floor(gy);
	fx = gx - flx;
	fy = gy - fly;
	// powers of two: the mask wraps x == L to node 0 and keeps every
	// index in range whatever the position
	ix = (int) flx & (g.nx - 1);
	iy = (int) fly & (g.ny - 1);
	ix1 = (ix + 1) & (g.nx - 1);
	iy1 = (iy + 1) & (g.ny - 1);
}

__device__ __forceinline__ void red_add(unsigned long long *a, long long v)
{
	atomicAdd(a, (unsigned long long) v);
}

__device__ __forceinline__ void max_bits(unsigned long long *a, double v)
{
	// non-negative doubles order like their bit patterns
	atomicMax(a, (unsigned long long) __double_as_longlong(fabs(v)));
}

template <typename T>
__device__ __forceinline__ T warp_max(T v)
{
	for(int o = 16; o > 0; o >>= 1)
		v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
	return v;
}

// ---------------------------------------------------------------- forward

template <typename T>
__device__ __forceinline__ void deposit_rho(const AGrid &g, T x, T y, double qfix,
		unsigned long long *rho)
{
	int ix, iy, ix1, iy1;
	T fx, fy;
	cell<T>(g, x, y, ix, iy, ix1, iy1, fx, fy);
	double w00 = (double) ((1 - fx) * (1 - fy)), w10 = (double) (fx * (1 - fy));
	double w01 = (double) ((1 - fx) * fy), w11 = (double) (fx * fy);
	red_add(rho + (int64_t) iy * g.nx + ix, __double2ll_rn(w00 * qfix));
	red_add(rho + (int64_t) iy * g.nx + ix1, __double2ll_rn(w10 * qfix));
	red_add(rho + (int64_t) iy1 * g.nx + ix, __double2ll_rn(w01 * qfix));
	red_add(rho + (int64_t) iy1 * g.nx + ix1, __double2ll_rn(w11 * qfix));
}

template <typename T>
__global__ void k_deposit(AGrid g, int64_t n, const T *x, const T *y, double qfix,
		unsigned long long *rho)
{
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
			i += (int64_t) gridDim.x * blockDim.x)
		deposit_rho<T>(g, x[i], y[i], qfix, rho);
}

// E = -grad phi by periodic central differences.
template <typename T>
__global__ void k_E(AGrid g, const T *phi, T *Ex, T *Ey)
{
	int64_t ng = (int64_t) g.nx * g.ny;
	T cx = (T) (0.5 * g.idx), cy = (T) (0.5 * g.idy);
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < ng;
			i += (int64_t) gridDim.x * blockDim.x)
	{
		int iy = (int) (i / g.nx), ix = (int) (i - (int64_t) iy * g.nx);
		int xm = (ix - 1) & (g.nx - 1), xp = (ix + 1) & (g.nx - 1);
		int ym = (iy - 1) & (g.ny - 1), yp = (iy + 1) & (g.ny - 1);
		Ex[i] = (phi[(int64_t) iy * g.nx + xm] - phi[(int64_t) iy * g.nx + xp]) * cx;
		Ey[i] = (phi[(int64_t) ym * g.nx + ix] - phi[(int64_t) yp * g.nx + ix]) * cy;
	}
}

// Gather, kick, move, wrap; deposit of the new position.  hx/hy (may be
// null) receive the positions before the move.
template <typename T>
__global__ void k_push(AGrid g, int64_t n, T *x, T *y, T *ux, T *uy, const T *Ex, const T *Ey,
		Kick k, T dt, double qfix, unsigned long long *rho, T *hx, T *hy)
{
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
			i += (int64_t) gridDim.x * blockDim.x)
	{
		T px = x[i], py = y[i];
		if(hx) { hx[i] = px; hy[i] = py; }
		int ix, iy, ix1, iy1;
		T fx, fy;
		cell<T>(g, px, py, ix, iy, ix1, iy1, fx, fy);
		int64_t n00 = (int64_t) iy * g.nx + ix, n10 = (int64_t) iy * g.nx + ix1;
		int64_t n01 = (int64_t) iy1 * g.nx + ix, n11 = (int64_t) iy1 * g.nx + ix1;
		T w00 = (1 - fx) * (1 - fy), w10 = fx * (1 - fy), w01 = (1 - fx) * fy, w11 = fx * fy;
		T ex = w00 * Ex[n00] + w10 * Ex[n10] + w01 * Ex[n01] + w11 * Ex[n11];
		T ey = w00 * Ey[n00] + w10 * Ey[n10] + w01 * Ey[n01] + w11 * Ey[n11];
		T h = (T) k.h, t = (T) k.t, s = (T) k.s;
		T vmx = ux[i] + h * ex, vmy = uy[i] + h * ey;
		T vpx = vmx + vmy * t, vpy = vmy - vmx * t;
		T vx = vmx + vpy * s + h * ex, vy = vmy - vpx * s + h * ey;
		ux[i] = vx;
		uy[i] = vy;
		if(k.move)
		{
			px += dt * vx;
			py += dt * vy;
			if(px >= (T) g.Lx) px -= (T) g.Lx;
			else if(px < 0) px += (T) g.Lx;
			if(py >= (T) g.Ly) py -= (T) g.Ly;
			else if(py < 0) py += (T) g.Ly;
			x[i] = px;
			y[i] = py;
		}
		deposit_rho<T>(g, px, py, qfix, rho);
	}
}

// Per-block partial sums of |E|^2 (FP64), then one block adds them in a
// fixed order: deterministic.
template <typename T>
__global__ void k_energy_part(int64_t ng, const T *Ex, const T *Ey, double *part)
{
	__shared__ double sh[32];
	double acc = 0.0;
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < ng;
			i += (int64_t) gridDim.x * blockDim.x)
	{
		double a = (double) Ex[i], b = (double) Ey[i];
		acc += a * a + b * b;
	}
	for(int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
	if((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
	__syncthreads();
	if(threadIdx.x == 0)
	{
		double s = 0.0;
		for(int w = 0; w < (int) (blockDim.x >> 5); w++) s += sh[w];
		part[blockIdx.x] = s;
	}
}

__global__ void k_sum_parts(int nb, const double *part, double scale, double *out)
{
	if(threadIdx.x == 0 && blockIdx.x == 0)
	{
		double s = 0.0;
		for(int b = 0; b < nb; b++) s += part[b];
		*out = s * scale;
	}
}

// Exact integer sum of the fixed-point charge (the k = 0 mode removed
// before an FP32 transform).  One block.
__global__ void k_isum(int64_t ng, const long long *rho, long long *out)
{
	__shared__ long long sh[32];
	long long acc = 0;
	for(int64_t i = threadIdx.x; i < ng; i += blockDim.x) acc += rho[i];
	for(int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
	if((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
	__syncthreads();
	if(threadIdx.x == 0)
	{
		long long s = 0;
		for(int w = 0; w < (int) (blockDim.x >> 5); w++) s += sh[w];
		*out = s;
	}
}

// ---------------------------------------------------------------- reverse

// Eb = e0 dx dy E (dL/dE of the loss).
template <typename T>
__global__ void k_loss_grad(int64_t ng, const T *Ex, const T *Ey, double f, T *Ebx, T *Eby)
{
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < ng;
			i += (int64_t) gridDim.x * blockDim.x)
	{
		Ebx[i] = (T) (f * (double) Ex[i]);
		Eby[i] = (T) (f * (double) Ey[i]);
	}
}

// Fixed-point Eb (two components) -> real.
template <typename T>
__global__ void k_fix_to_real(int64_t ng, const long long *bx, const long long *by,
		const Scale *sc, T *Ebx, T *Eby)
{
	double inv = sc->einv;
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < ng;
			i += (int64_t) gridDim.x * blockDim.x)
	{
		Ebx[i] = (T) ((double) bx[i] * inv);
		Eby[i] = (T) ((double) by[i] * inv);
	}
}

// phib = (-grad_h)^T Eb: phib_m = (Ebx[m+1] - Ebx[m-1]) / (2dx) + same in y.
template <typename T>
__global__ void k_div(AGrid g, const T *Ebx, const T *Eby, T *phib)
{
	int64_t ng = (int64_t) g.nx * g.ny;
	T cx = (T) (0.5 * g.idx), cy = (T) (0.5 * g.idy);
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < ng;
			i += (int64_t) gridDim.x * blockDim.x)
	{
		int iy = (int) (i / g.nx), ix = (int) (i - (int64_t) iy * g.nx);
		int xm = (ix - 1) & (g.nx - 1), xp = (ix + 1) & (g.nx - 1);
		int ym = (iy - 1) & (g.ny - 1), yp = (iy + 1) & (g.ny - 1);
		phib[i] = (Ebx[(int64_t) iy * g.nx + xp] - Ebx[(int64_t) iy * g.nx + xm]) * cx
			+ (Eby[(int64_t) yp * g.nx + ix] - Eby[(int64_t) ym * g.nx + ix]) * cy;
	}
}

// max |rhob| into sc->rmax.
template <typename T>
__global__ void k_absmax(int64_t ng, const T *v, Scale *sc)
{
	T m = 0;
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < ng;
			i += (int64_t) gridDim.x * blockDim.x)
		m = fmax(m, fabs(v[i]));
	m = warp_max<T>(m);
	if((threadIdx.x & 31) == 0) max_bits(&sc->rmax, (double) m);
}

// Scale of the next adjoint deposit from a bound on |eb|:
//   |ut|_inf <= umax + move dt (pmax + |c| 2 max(idx, idy) rmax)
//   |eb|_inf <= |h| (1 + |a| + |s|) |ut|_inf
// and a node sums at most n such contributions (weights sum to 1).
__global__ void k_scale(Scale *sc, Kick k, double dt, double c, double gmax, double n)
{
	if(threadIdx.x || blockIdx.x) return;
	// maxima of the previous reverse step's outputs
	sc->umax = sc->umax_n;
	sc->pmax = sc->pmax_n;
	sc->umax_n = 0;
	sc->pmax_n = 0;
	double umax = __longlong_as_double((long long) sc->umax);
	double pmax = __longlong_as_double((long long) sc->pmax);
	double rmax = __longlong_as_double((long long) sc->rmax);
	double ut = umax + (k.move ? dt * (pmax + fabs(c) * 2.0 * gmax * rmax) : 0.0);
	double eb = fabs(k.h) * (1.0 + fabs(k.a) + fabs(k.s)) * ut;
	double bound = n * eb;
	if(!(bound > 0.0) || !isfinite(bound))
	{
		sc->emul = 1.0;
		sc->einv = 1.0;
	}
	else
	{
		int e = (int) floor(62.0 - log2(bound)) - 1;
		sc->emul = ldexp(1.0, e);
		sc->einv = ldexp(1.0, -e);
	}
	sc->rmax = 0;
}

// grad of sum_n w_n(p) F_n with respect to p.
template <typename T>
__device__ __forceinline__ void wgrad(const AGrid &g, T fx, T fy, T f00, T f10, T f01, T f11,
		T &gx, T &gy)
{
	gx = (T) g.idx * ((1 - fy) * (f10 - f00) + fy * (f11 - f01));
	gy = (T) g.idy * ((1 - fx) * (f01 - f00) + fx * (f11 - f10));
}

// One reverse step j, fused with the deposit term of step j+1 (nxt = p_{j+1},
// rhob = rhob_{j+1}; nxt null: that term was already added).
template <typename T>
__global__ void k_rev(AGrid g, int64_t n, const T *nx_, const T *ny_, const T *rhob, double c,
		const T *px_, const T *py_, const T *Ex, const T *Ey, Kick k, T dt, T *pbx, T *pby,
		T *ubx, T *uby, Scale *sc, unsigned long long *Ebx, unsigned long long *Eby)
{
	double emul = sc->emul;
	T umax = 0, pmax = 0;
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
			i += (int64_t) gridDim.x * blockDim.x)
	{
		T bx = pbx[i], by = pby[i];
		int ix, iy, ix1, iy1;
		T fx, fy, gx, gy;
		if(nx_)
		{
			cell<T>(g, nx_[i], ny_[i], ix, iy, ix1, iy1, fx, fy);
			wgrad<T>(g, fx, fy, rhob[(int64_t) iy * g.nx + ix], rhob[(int64_t) iy * g.nx + ix1],
					rhob[(int64_t) iy1 * g.nx + ix], rhob[(int64_t) iy1 * g.nx + ix1], gx, gy);
			bx += (T) c * gx;
			by += (T) c * gy;
		}
		T utx = ubx[i], uty = uby[i];
		if(k.move) { utx += dt * bx; uty += dt * by; }
		T a = (T) k.a, s = (T) k.s, h = (T) k.h;
		T vbx = a * utx - s * uty, vby = s * utx + a * uty;
		T ebx = h * (utx + vbx), eby = h * (uty + vby);
		cell<T>(g, px_[i], py_[i], ix, iy, ix1, iy1, fx, fy);
		int64_t n00 = (int64_t) iy * g.nx + ix, n10 = (int64_t) iy * g.nx + ix1;
		int64_t n01 = (int64_t) iy1 * g.nx + ix, n11 = (int64_t) iy1 * g.nx + ix1;
		T d00 = Ex[n00] * ebx + Ey[n00] * eby, d10 = Ex[n10] * ebx + Ey[n10] * eby;
		T d01 = Ex[n01] * ebx + Ey[n01] * eby, d11 = Ex[n11] * ebx + Ey[n11] * eby;
		wgrad<T>(g, fx, fy, d00, d10, d01, d11, gx, gy);
		bx += gx;
		by += gy;
		pbx[i] = bx;
		pby[i] = by;
		ubx[i] = vbx;
		uby[i] = vby;
		umax = fmax(umax, fmax(fabs(vbx), fabs(vby)));
		pmax = fmax(pmax, fmax(fabs(bx), fabs(by)));
		double w00 = (double) ((1 - fx) * (1 - fy)), w10 = (double) (fx * (1 - fy));
		double w01 = (double) ((1 - fx) * fy), w11 = (double) (fx * fy);
		double ex = (double) ebx * emul, ey = (double) eby * emul;
		red_add(Ebx + n00, __double2ll_rn(w00 * ex));
		red_add(Ebx + n10, __double2ll_rn(w10 * ex));
		red_add(Ebx + n01, __double2ll_rn(w01 * ex));
		red_add(Ebx + n11, __double2ll_rn(w11 * ex));
		red_add(Eby + n00, __double2ll_rn(w00 * ey));
		red_add(Eby + n10, __double2ll_rn(w10 * ey));
		red_add(Eby + n01, __double2ll_rn(w01 * ey));
		red_add(Eby + n11, __double2ll_rn(w11 * ey));
	}
	umax = warp_max<T>(umax);
	pmax = warp_max<T>(pmax);
	if((threadIdx.x & 31) == 0)
	{
		max_bits(&sc->umax_n, (double) umax);
		max_bits(&sc->pmax_n, (double) pmax);
	}
}

// Last term: pb_0 += c grad D(p_0)^T rhob_0; results to FP64.
template <typename T>
__global__ void k_finish(AGrid g, int64_t n, const T *px_, const T *py_, const T *rhob, double c,
		const T *pbx, const T *pby, const T *ubx, const T *uby, double *out)
{
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
			i += (int64_t) gridDim.x * blockDim.x)
	{
		int ix, iy, ix1, iy1;
		T fx, fy, gx, gy;
		cell<T>(g, px_[i], py_[i], ix, iy, ix1, iy1, fx, fy);
		wgrad<T>(g, fx, fy, rhob[(int64_t) iy * g.nx + ix], rhob[(int64_t) iy * g.nx + ix1],
				rhob[(int64_t) iy1 * g.nx + ix], rhob[(int64_t) iy1 * g.nx + ix1], gx, gy);
		out[i] = (double) pbx[i] + c * (double) gx;
		out[n + i] = (double) pby[i] + c * (double) gy;
		out[2 * n + i] = (double) ubx[i];
		out[3 * n + i] = (double) uby[i];
	}
}

template <typename T>
__global__ void k_from_f64(int64_t n, const double *in, T *out)
{
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
			i += (int64_t) gridDim.x * blockDim.x)
		out[i] = (T) in[i];
}

} // namespace adj
} // namespace cpic

using namespace cpic;
using namespace cpic::adj;

struct cpic_adj {
	cpic_adj_params_t p;
	AGrid g;
	Grid fg;                  // for the FFT launchers (nx, ny)
	int64_t n, ng;
	bool f64;
	size_t ts;                // sizeof(T)
	double qfix, qinv;        // forward charge fixed point
	cudaStream_t st;
	cudaEvent_t ev[4];
	// particles (T): x, y, ux, uy; adjoints pbx, pby, ubx, uby
	void *x, *y, *ux, *uy, *pbx, *pby, *ubx, *uby;
	void *ckpt;               // nckpt x 4 x n (T)
	void *hist;               // K x 2 x n (T): positions p_j of a segment
	void *histE;              // K x 2 x ng (T): fields E_j of a segment
	void *Ex, *Ey;            // current field (T)
	void *phi, *rhob, *Ebx, *Eby, *spec;
	long long *rho, *Ebfix;   // ng; 2 x ng
	long long *rsum;
	Scale *sc;
	double *part, *loss_d, *stage;
	void *twx, *twy;
	double *cosx, *cosy;
	int nckpt;
	bool have_forward;
	double loss;
	float ms_fwd, ms_bwd;
};

namespace {

int blocks_for(int64_t n)
{
	int64_t b = (n + 255) / 256;
	if(b > 152 * 16) b = 152 * 16;
	return (int) (b < 1 ? 1 : b);
}

Kick kick_of(const cpic_adj *a, int64_t j)
{
	Kick k;
	double dtp = j == 0 ? -0.5 * a->p.dt : a->p.dt;   // mover.c:204-213
	k.h = 0.5 * dtp * a->p.q / a->p.m;
	k.t = a->p.Bz * k.h;
	k.s = 2.0 * k.t / (1.0 + k.t * k.t);
	k.a = 1.0 - k.s * k.t;
	k.move = j == 0 ? 0 : 1;
	return k;
}

template <typename T>
T *P(void *v, int64_t off = 0) { return reinterpret_cast<T *>(v) + off; }

// rho (fixed point) -> E (T) into Ex/Ey.
template <typename T>
void solve_E(cpic_adj *a, T *Ex, T *Ey)
{
	typedef typename Cx<T>::t C;
	const long long *mean = nullptr;
	if(!a->f64)
	{
		k_isum<<<1, 1024, 0, a->st>>>(a->ng, a->rho, a->rsum);
		mean = a->rsum;
	}
	poisson_launch<T>(a->fg, a->rho, a->qinv, mean, P<C>(a->spec), P<C>(a->twx), P<C>(a->twy),
			a->cosx, a->cosy, P<T>(a->phi), a->st);
	k_E<T><<<blocks_for(a->ng), 256, 0, a->st>>>(a->g, P<T>(a->phi), Ex, Ey);
}

// Steps [j0, j1) from the current state; hist != 0: keep p_j and E_j.
template <typename T>
void run_steps(cpic_adj *a, int64_t j0, int64_t j1, bool hist, bool ckpt)
{
	int64_t n = a->n, ng = a->ng;
	int K = (int) a->p.checkpoint_every;
	for(int64_t j = j0; j < j1; j++)
	{
		if(ckpt && j % K == 0)
		{
			T *c = P<T>(a->ckpt, (j / K) * 4 * n);
			cudaMemcpyAsync(c, a->x, n * sizeof(T), cudaMemcpyDeviceToDevice, a->st);
			cudaMemcpyAsync(c + n, a->y, n * sizeof(T), cudaMemcpyDeviceToDevice, a->st);
			cudaMemcpyAsync(c + 2 * n, a->ux, n * sizeof(T), cudaMemcpyDeviceToDevice, a->st);
			cudaMemcpyAsync(c + 3 * n, a->uy, n * sizeof(T), cudaMemcpyDeviceToDevice, a->st);
		}
		int64_t s = j - j0;
		T *Ex = hist ? P<T>(a->histE, s * 2 * ng) : P<T>(a->Ex);
		T *Ey = hist ? Ex + ng : P<T>(a->Ey);
		solve_E<T>(a, Ex, Ey);
		cudaMemsetAsync(a->rho, 0, ng * sizeof(long long), a->st);
		T *hx = hist ? P<T>(a->hist, s * 2 * n) : nullptr;
		T *hy = hist ? hx + n : nullptr;
		k_push<T><<<blocks_for(n), 256, 0, a->st>>>(a->g, n, P<T>(a->x), P<T>(a->y), P<T>(a->ux),
				P<T>(a->uy), Ex, Ey, kick_of(a, j), (T) a->p.dt, a->qfix,
				reinterpret_cast<unsigned long long *>(a->rho), hx, hy);
	}
}

// Eb (T, in a->Ebx/Eby) -> rhob; and its max into sc->rmax.
template <typename T>
void grid_adjoint(cpic_adj *a)
{
	typedef typename Cx<T>::t C;
	k_div<T><<<blocks_for(a->ng), 256, 0, a->st>>>(a->g, P<T>(a->Ebx), P<T>(a->Eby), P<T>(a->phi));
	poisson_launch_real<T>(a->fg, P<T>(a->phi), P<C>(a->spec), P<C>(a->twx), P<C>(a->twy),
			a->cosx, a->cosy, P<T>(a->rhob), a->st);
	k_absmax<T><<<blocks_for(a->ng), 256, 0, a->st>>>(a->ng, P<T>(a->rhob), a->sc);
}

template <typename T>
int forward_impl(cpic_adj *a)
{
	int64_t n = a->n, ng = a->ng;
	cudaEventRecord(a->ev[0], a->st);
	cudaMemsetAsync(a->rho, 0, ng * sizeof(long long), a->st);
	k_deposit<T><<<blocks_for(n), 256, 0, a->st>>>(a->g, n, P<T>(a->x), P<T>(a->y), a->qfix,
			reinterpret_cast<unsigned long long *>(a->rho));
	run_steps<T>(a, 0, a->p.nsteps, false, true);
	solve_E<T>(a, P<T>(a->Ex), P<T>(a->Ey));
	int nb = 152;
	k_energy_part<T><<<nb, 256, 0, a->st>>>(ng, P<T>(a->Ex), P<T>(a->Ey), a->part);
	k_sum_parts<<<1, 32, 0, a->st>>>(nb, a->part, 0.5 * a->p.e0 * a->g.dx * a->g.dy, a->loss_d);
	cudaEventRecord(a->ev[1], a->st);
	cudaMemcpyAsync(&a->loss, a->loss_d, sizeof(double), cudaMemcpyDeviceToHost, a->st);
	if(cudaStreamSynchronize(a->st) != cudaSuccess) return CPIC_ECUDA;
	cudaEventElapsedTime(&a->ms_fwd, a->ev[0], a->ev[1]);
	return CPIC_OK;
}

template <typename T>
int backward_impl(cpic_adj *a)
{
	int64_t n = a->n, ng = a->ng, N = a->p.nsteps;
	int K = (int) a->p.checkpoint_every;
	double c = -a->p.q / a->p.e0;                 // interpolate.c:307
	double gmax = a->g.idx > a->g.idy ? a->g.idx : a->g.idy;
	cudaEventRecord(a->ev[2], a->st);
	// dL/dE of the final field (a->Ex/Ey still hold it), then rhob_N
	k_loss_grad<T><<<blocks_for(ng), 256, 0, a->st>>>(ng, P<T>(a->Ex), P<T>(a->Ey),
			a->p.e0 * a->g.dx * a->g.dy, P<T>(a->Ebx), P<T>(a->Eby));
	cudaMemsetAsync(a->sc, 0, sizeof(Scale), a->st);
	grid_adjoint<T>(a);
	cudaMemsetAsync(a->pbx, 0, n * sizeof(T), a->st);
	cudaMemsetAsync(a->pby, 0, n * sizeof(T), a->st);
	cudaMemsetAsync(a->ubx, 0, n * sizeof(T), a->st);
	cudaMemsetAsync(a->uby, 0, n * sizeof(T), a->st);
	int64_t nseg = (N + K - 1) / K;
	bool have_next = true;      // the deposit term of p_N is still to add
	for(int64_t sgi = nseg - 1; sgi >= 0; sgi--)
	{
		int64_t j0 = sgi * K, j1 = j0 + K < N ? j0 + K : N;
		// restore the checkpoint and recompute the segment
		T *ck = P<T>(a->ckpt, sgi * 4 * n);
		cudaMemcpyAsync(a->x, ck, n * sizeof(T), cudaMemcpyDeviceToDevice, a->st);
		cudaMemcpyAsync(a->y, ck + n, n * sizeof(T), cudaMemcpyDeviceToDevice, a->st);
		cudaMemcpyAsync(a->ux, ck + 2 * n, n * sizeof(T), cudaMemcpyDeviceToDevice, a->st);
		cudaMemcpyAsync(a->uy, ck + 3 * n, n * sizeof(T), cudaMemcpyDeviceToDevice, a->st);
		cudaMemsetAsync(a->rho, 0, ng * sizeof(long long), a->st);
		k_deposit<T><<<blocks_for(n), 256, 0, a->st>>>(a->g, n, P<T>(a->x), P<T>(a->y), a->qfix,
				reinterpret_cast<unsigned long long *>(a->rho));
		run_steps<T>(a, j0, j1, true, false);
		// after the recompute a->x/y hold p_{j1}
		for(int64_t j = j1 - 1; j >= j0; j--)
		{
			int64_t s = j - j0;
			const T *nxp, *nyp;
			if(j + 1 == j1) { nxp = P<T>(a->x); nyp = P<T>(a->y); }
			else { nxp = P<T>(a->hist, (s + 1) * 2 * n); nyp = nxp + n; }
			Kick k = kick_of(a, j);
			k_scale<<<1, 32, 0, a->st>>>(a->sc, k, a->p.dt, c, gmax, (double) n);
			cudaMemsetAsync(a->Ebfix, 0, 2 * ng * sizeof(long long), a->st);
			const T *hp = P<T>(a->hist, s * 2 * n);
			const T *hE = P<T>(a->histE, s * 2 * ng);
			k_rev<T><<<blocks_for(n), 256, 0, a->st>>>(a->g, n, have_next ? nxp : nullptr,
					have_next ? nyp : nullptr, P<T>(a->rhob), c, hp, hp + n, hE, hE + ng, k,
					(T) a->p.dt, P<T>(a->pbx), P<T>(a->pby), P<T>(a->ubx), P<T>(a->uby), a->sc,
					reinterpret_cast<unsigned long long *>(a->Ebfix),
					reinterpret_cast<unsigned long long *>(a->Ebfix + ng));
			have_next = true;
			k_fix_to_real<T><<<blocks_for(ng), 256, 0, a->st>>>(ng, a->Ebfix, a->Ebfix + ng, a->sc,
					P<T>(a->Ebx), P<T>(a->Eby));
			grid_adjoint<T>(a);
		}
	}
	// pb_0 += c grad D(p_0)^T rhob_0 (p_0 = the first checkpoint)
	T *p0 = P<T>(a->ckpt);
	k_finish<T><<<blocks_for(n), 256, 0, a->st>>>(a->g, n, p0, p0 + n, P<T>(a->rhob), c,
			P<T>(a->pbx), P<T>(a->pby), P<T>(a->ubx), P<T>(a->uby), a->stage);
	cudaEventRecord(a->ev[3], a->st);
	if(cudaStreamSynchronize(a->st) != cudaSuccess) return CPIC_ECUDA;
	cudaEventElapsedTime(&a->ms_bwd, a->ev[2], a->ev[3]);
	return CPIC_OK;
}

bool pow2i(int64_t v) { return v >= 4 && (v & (v - 1)) == 0; }

} // namespace

CPIC_API int cpic_adj_create(const cpic_adj_params_t *p, int64_t n, cpic_adj_t **out)
{
	if(!p || !out || n <= 0) return CPIC_EINVAL;
	*out = nullptr;
	if(!pow2i(p->nx) || !pow2i(p->ny) || p->nx > 16384 || p->ny > 16384) return CPIC_EINVAL;
	if(!(p->Lx > 0) || !(p->Ly > 0) || !(p->dt > 0) || !(p->e0 > 0) || p->m == 0.0 || p->q == 0.0)
		return CPIC_EINVAL;
	if(p->nsteps < 1 || p->checkpoint_every < 1) return CPIC_EINVAL;
	if(p->precision != CPIC_FP64 && p->precision != CPIC_MIXED) return CPIC_EINVAL;
	int ndev = 0;
	if(cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return CPIC_ENODEV;

	cpic_adj *a = new cpic_adj();
	a->p = *p;
	if(a->p.checkpoint_every > a->p.nsteps) a->p.checkpoint_every = a->p.nsteps;
	a->n = n;
	a->g.nx = (int) p->nx; a->g.ny = (int) p->ny;
	a->g.Lx = p->Lx; a->g.Ly = p->Ly;
	a->g.dx = p->Lx / p->nx; a->g.dy = p->Ly / p->ny;
	a->g.idx = 1.0 / a->g.dx; a->g.idy = 1.0 / a->g.dy;
	memset(&a->fg, 0, sizeof(a->fg));
	a->fg.nx = a->g.nx; a->fg.ny = a->g.ny;
	a->ng = p->nx * p->ny;
	a->f64 = p->precision == CPIC_FP64;
	a->ts = a->f64 ? sizeof(double) : sizeof(float);
	// |rho| sums at most n |q/e0| (weights sum to 1): no wrap below 2^62
	double bound = (double) n * fabs(p->q / p->e0);
	int k = (int) floor(62.0 - log2(bound)) - 1;
	a->qfix = -p->q / p->e0 * ldexp(1.0, k);
	a->qinv = ldexp(1.0, -k);
	int K = (int) a->p.checkpoint_every;
	a->nckpt = (int) ((p->nsteps + K - 1) / K);
	int64_t ng = a->ng, nh = p->nx / 2 + 1;
	size_t ts = a->ts, cs = 2 * ts;
	int r = CPIC_OK;
	if(cudaStreamCreateWithFlags(&a->st, cudaStreamNonBlocking) != cudaSuccess)
	{
		delete a;
		return CPIC_ECUDA;
	}
	for(int i = 0; i < 4; i++) cudaEventCreate(&a->ev[i]);
#define AL(ptr, bytes) do { if(cudaMalloc((void **) &(ptr), (bytes)) != cudaSuccess) { r = CPIC_ENOMEM; goto fail; } } while(0)
	AL(a->x, n * ts); AL(a->y, n * ts); AL(a->ux, n * ts); AL(a->uy, n * ts);
	AL(a->pbx, n * ts); AL(a->pby, n * ts); AL(a->ubx, n * ts); AL(a->uby, n * ts);
	AL(a->ckpt, (size_t) a->nckpt * 4 * n * ts);
	AL(a->hist, (size_t) K * 2 * n * ts);
	AL(a->histE, (size_t) K * 2 * ng * ts);
	AL(a->Ex, ng * ts); AL(a->Ey, ng * ts);
	AL(a->phi, ng * ts); AL(a->rhob, ng * ts); AL(a->Ebx, ng * ts); AL(a->Eby, ng * ts);
	AL(a->spec, (size_t) p->ny * nh * cs);
	AL(a->rho, ng * sizeof(long long));
	AL(a->Ebfix, 2 * ng * sizeof(long long));
	AL(a->rsum, sizeof(long long));
	AL(a->sc, sizeof(Scale));
	AL(a->part, 152 * sizeof(double));
	AL(a->loss_d, sizeof(double));
	AL(a->stage, 4 * n * sizeof(double));
	AL(a->twx, p->nx / 2 * cs); AL(a->twy, p->ny / 2 * cs);
	AL(a->cosx, p->nx * sizeof(double)); AL(a->cosy, p->ny * sizeof(double));
#undef AL
	{
		// Green's function cosines (solver.c:257-278) and twiddles, as the
		// step's own solver builds them
		std::vector<double> cx(p->nx), cy(p->ny);
		for(int64_t i = 0; i < p->nx; i++) cx[i] = cos(2.0 * M_PI / p->nx * i);
		for(int64_t i = 0; i < p->ny; i++) cy[i] = cos(2.0 * M_PI / p->ny * i);
		cudaMemcpy(a->cosx, cx.data(), p->nx * sizeof(double), cudaMemcpyHostToDevice);
		cudaMemcpy(a->cosy, cy.data(), p->ny * sizeof(double), cudaMemcpyHostToDevice);
		for(int dim = 0; dim < 2; dim++)
		{
			int64_t m = dim == 0 ? p->nx : p->ny;
			std::vector<double2> tw(m / 2);
			std::vector<float2> tf(m / 2);
			for(int64_t i = 0; i < m / 2; i++)
			{
				double ang = -2.0 * M_PI * i / m;
				tw[i] = make_double2(cos(ang), sin(ang));
				tf[i] = make_float2((float) cos(ang), (float) sin(ang));
			}
			void *dst = dim == 0 ? a->twx : a->twy;
			if(a->f64) cudaMemcpy(dst, tw.data(), m / 2 * sizeof(double2), cudaMemcpyHostToDevice);
			else cudaMemcpy(dst, tf.data(), m / 2 * sizeof(float2), cudaMemcpyHostToDevice);
		}
	}
	{
		static PerDeviceOnce once;
		cudaError_t e = once.run([] {
			return set_max_dyn_smem({(const void *) k_rows_fwd<double>, (const void *) k_cols<double>,
					(const void *) k_rows_inv<double>, (const void *) k_rows_fwd_real<double>,
					(const void *) k_rows_fwd<float>, (const void *) k_cols<float>,
					(const void *) k_rows_inv<float>, (const void *) k_rows_fwd_real<float>},
					200 * 1024);
		});
		if(e != cudaSuccess)
		{
			fprintf(stderr, "cpic_adj_create: kernel set-up failed: %s\n", cudaGetErrorString(e));
			r = CPIC_ECUDA;
			goto fail;
		}
	}
	if(cudaDeviceSynchronize() != cudaSuccess) { r = CPIC_ECUDA; goto fail; }
	*out = a;
	return CPIC_OK;
fail:
	cpic_adj_destroy(a);
	return r;
}

CPIC_API void cpic_adj_destroy(cpic_adj_t *a)
{
	if(!a) return;
	void *bufs[] = {a->x, a->y, a->ux, a->uy, a->pbx, a->pby, a->ubx, a->uby, a->ckpt, a->hist,
		a->histE, a->Ex, a->Ey, a->phi, a->rhob, a->Ebx, a->Eby, a->spec, a->rho, a->Ebfix,
		a->rsum, a->sc, a->part, a->loss_d, a->stage, a->twx, a->twy, a->cosx, a->cosy};
	for(void *b : bufs) if(b) cudaFree(b);
	for(int i = 0; i < 4; i++) if(a->ev[i]) cudaEventDestroy(a->ev[i]);
	if(a->st) cudaStreamDestroy(a->st);
	delete a;
}

CPIC_API int cpic_adj_forward(cpic_adj_t *a, const double *x, const double *y, const double *ux,
		const double *uy, double *loss)
{
	if(!a || !x || !y || !ux || !uy) return CPIC_EINVAL;
	int64_t n = a->n;
	for(int64_t i = 0; i < n; i++)
	{
		if(!(x[i] >= 0.0 && x[i] < a->p.Lx && y[i] >= 0.0 && y[i] < a->p.Ly)) return CPIC_EINVAL;
		if(!std::isfinite(ux[i]) || !std::isfinite(uy[i])) return CPIC_EINVAL;
	}
	const double *src[4] = {x, y, ux, uy};
	void *dst[4] = {a->x, a->y, a->ux, a->uy};
	for(int c = 0; c < 4; c++)
	{
		if(cudaMemcpyAsync(a->stage, src[c], n * sizeof(double), cudaMemcpyHostToDevice, a->st)
				!= cudaSuccess)
			return CPIC_ECUDA;
		if(a->f64) k_from_f64<double><<<blocks_for(n), 256, 0, a->st>>>(n, a->stage, (double *) dst[c]);
		else k_from_f64<float><<<blocks_for(n), 256, 0, a->st>>>(n, a->stage, (float *) dst[c]);
	}
	int r = a->f64 ? forward_impl<double>(a) : forward_impl<float>(a);
	if(r) return r;
	if(cudaGetLastError() != cudaSuccess) return CPIC_ECUDA;
	a->have_forward = true;
	if(loss) *loss = a->loss;
	return CPIC_OK;
}

CPIC_API int cpic_adj_backward(cpic_adj_t *a, double *gx, double *gy, double *gux, double *guy)
{
	if(!a) return CPIC_EINVAL;
	if(!a->have_forward) return CPIC_ESTATE;
	int r = a->f64 ? backward_impl<double>(a) : backward_impl<float>(a);
	if(r) return r;
	if(cudaGetLastError() != cudaSuccess) return CPIC_ECUDA;
	// the forward state was overwritten by the recompute: a new forward is
	// needed before the next backward
	a->have_forward = false;
	double *outs[4] = {gx, gy, gux, guy};
	int64_t n = a->n;
	for(int c = 0; c < 4; c++)
		if(outs[c] && cudaMemcpy(outs[c], a->stage + c * n, n * sizeof(double),
					cudaMemcpyDeviceToHost) != cudaSuccess)
			return CPIC_ECUDA;
	return CPIC_OK;
}

CPIC_API int cpic_adj_times(const cpic_adj_t *a, double *ms_forward, double *ms_backward)
{
	if(!a) return CPIC_EINVAL;
	if(ms_forward) *ms_forward = a->ms_fwd;
	if(ms_backward) *ms_backward = a->ms_bwd;
	return CPIC_OK;
}
