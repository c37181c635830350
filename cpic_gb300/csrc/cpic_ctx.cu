// cpic_ctx.cu -- host context and C ABI (include/cpic_gpu.h), plus the
// generic device kernels: the merge of pending arrivals into the main
// regions, counting-sort rebuild of the particle store, host views and FP64
// diagnostics.
//
// Compiled with --fmad=false: the tile of an FP64 particle computed here
// must agree bit for bit with the one the push kernel computes.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#include <mutex>
#include <cudaTypedefs.h>   // PFN_cuTensorMapEncodeTiled

#include "../../include/cpic_gpu.h"
#include "cpic_common.cuh"
#include "cpic_push.cuh"
#include "cpic_fft.cuh"

namespace cpic {
void launch_gather_f64_tiles(const Grid &g, const StoreF64 &st, const int64_t *base,
		const int32_t *cnt, int ntiles, const double *Ex, const double *Ey,
		double *ex_out, double *ey_out, cudaStream_t s);
void launch_gather_mix_tiles(const Grid &g, const StoreMix &st, const int64_t *base,
		const int32_t *cnt, int ntiles, const float2 *E, double *ex_out, double *ey_out,
		cudaStream_t s);
}

using namespace cpic;

#define CK(call) do { cudaError_t e_ = (call); if(e_ != cudaSuccess) { \
	fprintf(stderr, "cpic: %s failed: %s (%s:%d)\n", #call, cudaGetErrorString(e_), \
		__FILE__, __LINE__); return CPIC_ECUDA; } } while(0)

// ------------------------------------------------------------- context

struct SpeciesHost {
	double q, m;
	int64_t n;
	int64_t cap_main, cap_alt;  // slots allocated in the store and its alternate
	StoreF64 f64, f64_alt;
	StoreMix mix, mix_alt;
	Tiles tiles;
	Spill spill[2];          // ping-pong: spill[cur] is the input
	double vmax;              // largest initial |u| component
	double wq_mult;           // mixed form: fixed-point units per weight unit
};

struct cpic_ctx {
	cpic_params_t p;
	Grid g;
	int ntiles;
	int ppt;                  // particles per thread of the fused kernel's instance
	int precision;
	int64_t iter;
	bool prepared;
	int slack_pct;            // tile capacity slack %, grows after overflows
	int64_t rebuilds;         // layout rebuilds forced by overflows
	int64_t last_spill;       // overflow records seen at the last check
	double qscale, qinv;
	double qlo_mul, qinv_lo;  // FP64 form: remainder-word scales
	bool wq_exact;            // mixed form: integer charge multiples
	cudaStream_t stream;
	int order_mode;           // tile order: 0 undecided, 1 computed each step, 2 kept
	int nspecies;
	SpeciesHost sp[kMaxSpecies];
	// parity of the double-buffered spill lists and arrivals buffers: the
	// next particle stage reads spill[spill_cur] and arrivals buffer
	// spill_cur, and writes the other ones
	int spill_cur;
	// fields
	long long *rho;           // ny x nx fixed point
	long long *rho_lo;        // FP64 form: remainder word (else null)
	double *phi64, *Ex64, *Ey64;
	float *phi32;
	float2 *E32;
	double2 *spec64;
	float2 *spec32;
	double2 *twx64, *twy64;
	float2 *twx32, *twy32;
	double *cosx, *cosy;
	double *green64;          // Green's function, column order (FP64 form)
	float *green32;           // same, FP32 (mixed form)
	double *mean;             // device scalar (mixed form)
	uint32_t *status;
	double *scratch;          // FP64 scratch for host views / partial sums
	size_t scratch_n;
	int32_t *counter;         // device scalar
	int32_t *probe_h;         // pinned: status word and each species' spill count
	CUtensorMap emap;         // mixed form: E32 as 2D tiles for the fused kernel
	bool emap_ok;
	unsigned long long *counter_pair;  // two device scalars (upload check)
};

// ------------------------------------------------------------- kernels

// Moves the arrivals in buffer a.arr_r into each tile's main region, so that
// every pass over the main regions sees all the species' particles (before a
// host read or a re-layout).  A tile whose main region has no room for all
// of them keeps them where they are and is counted in *overflow (the host
// then rebuilds the layout, which takes pending arrivals as they lie).
template <class F>
__global__ void k_merge(const PushArgs a, int32_t *overflow)
{
	const int s = blockIdx.y, t = blockIdx.x;
	const Tiles &T = a.tiles[s];
	const int r = a.arr_r;
	const int na = min(T.acnt[r][t], T.acap[t]), nm = T.cnt[t];
	if(na == 0)
		return;
	if(na > T.cap[t] - nm)
	{
		if(threadIdx.x == 0)
			atomicAdd(overflow, 1);
		return;
	}
	const int64_t src = T.abase[t] + (r ? T.abuf1 : 0), dst = T.base[t] + nm;
	for(int i = threadIdx.x; i < na; i += blockDim.x)
		F::store(a, s, dst + i, F::load(a, s, src + i));
	__syncthreads();
	if(threadIdx.x == 0)
	{
		T.cnt[t] = nm + na;
		T.acnt[r][t] = 0;
	}
}

// The order in which the next fused-kernel launch takes its tiles.  The
// hardware dispatches blocks in index order, one block per tile (4096
// tiles at 6 blocks per SM are about 4.5 waves); when the plasma bunches, a heavy tile
// dispatched late leaves most SMs idle while it finishes.  So tiles above
// 1.1x the mean count go first and tiles below 0.9x the mean go last, each
// group heaviest first in steps of 1/16 of the mean; the rest keep tile
// order in between, so a uniform plasma keeps the identity order (and
// neighbouring tiles, which write into each other's arrivals, run
// together).  A tile's count is its main region's plus the arrivals in
// buffer abuf (what the next launch reads).  A stable counting sort, so the
// order is a function of the counts alone.  Which block takes which tile
// changes no result.
constexpr int kOrderKeys = 512;
constexpr int kOrderMid = kOrderKeys - 1 - 255;      // bucket of the middle class
constexpr int kOrderThreads = 1024;
constexpr int kOrderMaxTiles = 8192;                 // larger layouts keep tile order
constexpr int kOrderPer = kOrderMaxTiles / kOrderThreads;

__device__ __forceinline__ int order_bucket(int32_t cnt, int ntiles, long long sum)
{
	long long c = (long long) cnt * ntiles;     // cnt / mean = c / sum
	int key;
	if(10 * c > 11 * sum)
		key = 256 + (int) min(255LL, 16 * c / sum);
	else if(10 * c < 9 * sum)
		key = (int) min(255LL, 16 * c / sum);
	else
		key = 255;
	return kOrderKeys - 1 - key;                 // larger keys first
}

// One block of kOrderThreads per species: the counts are read once, in
// parallel; a uniform layout (every tile in the middle class) writes the
// identity at once; otherwise warp 0 scans the bucket counts and scatters
// from the buckets kept in shared memory.
__global__ void __launch_bounds__(kOrderThreads) k_tile_order(const PushArgs a, int ntiles, int abuf)
{
	const Tiles &T = a.tiles[blockIdx.x];
	__shared__ uint16_t s_b[kOrderMaxTiles];
	__shared__ int32_t cur[kOrderKeys];
	__shared__ long long s_part[kOrderThreads / 32];
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	int32_t c[kOrderPer];
	long long sum = 0;
	#pragma unroll
	for(int k = 0; k < kOrderPer; k++)
	{
		const int i = k * kOrderThreads + tid;
		c[k] = i < ntiles ? T.cnt[i] + T.acnt[abuf][i] : 0;
		sum += c[k];
	}
	for(int o = 16; o > 0; o >>= 1)
		sum += __shfl_xor_sync(0xffffffffu, sum, o);
	if(lane == 0)
		s_part[warp] = sum;
	for(int k = tid; k < kOrderKeys; k += kOrderThreads)
		cur[k] = 0;
	__syncthreads();
	sum = 0;
	for(int w = 0; w < kOrderThreads / 32; w++)
		sum += s_part[w];
	int moved = 0;
	#pragma unroll
	for(int k = 0; k < kOrderPer; k++)
	{
		const int i = k * kOrderThreads + tid;
		if(i < ntiles)
		{
			const int b = sum > 0 ? order_bucket(c[k], ntiles, sum) : kOrderMid;
			s_b[i] = (uint16_t) b;
			moved |= b != kOrderMid;
			atomicAdd(&cur[b], 1);
		}
	}
	if(!__syncthreads_or(moved))
	{
		for(int i = tid; i < ntiles; i += kOrderThreads)
			T.order[i] = i;
		return;
	}
	if(warp != 0)
		return;
	// exclusive scan: lane l owns buckets [16 l, 16 l + 16)
	constexpr int per = kOrderKeys / 32;
	int loc = 0;
	for(int k = 0; k < per; k++)
		loc += cur[lane * per + k];
	int inc = loc;
	for(int o = 1; o < 32; o <<= 1)
	{
		int v = __shfl_up_sync(0xffffffffu, inc, o);
		if(lane >= o) inc += v;
	}
	int run = inc - loc;
	for(int k = 0; k < per; k++)
	{
		int v = cur[lane * per + k];
		cur[lane * per + k] = run;
		run += v;
	}
	__syncwarp();
	// stable scatter, 32 tiles at a time in tile order
	for(int i0 = 0; i0 < ntiles; i0 += 32)
	{
		const int i = i0 + lane;
		const int b = i < ntiles ? (int) s_b[i] : -1;
		const unsigned peers = __match_any_sync(0xffffffffu, b);
		const int pos = b >= 0 ? cur[b] + __popc(peers & lanemask_lt()) : 0;
		__syncwarp();
		if(b >= 0)
		{
			if(pos < ntiles)
				T.order[pos] = i;
			else
				set_status(a.status, ST_RANGE);
			if((peers & lanemask_lt()) == 0)
				cur[b] += __popc(peers);
		}
		__syncwarp();
	}
}

// Tile of a record given in the FP64 spill layout.
template <class F> struct TileOf;
template <> struct TileOf<F64> {
	static __device__ __forceinline__ int get(const Grid &g, const Spill &S, int64_t k)
	{
		double w[4];
		int cx, cy;
		F64::weights(g, S.x[k], S.y[k], w, cx, cy);
		cx = min(max(cx, 0), g.nx - 1);
		cy = min(max(cy, 0), g.ny - 1);
		return tile_of(g, cx, cy);
	}
};
template <> struct TileOf<Mix> {
	static __device__ __forceinline__ int get(const Grid &g, const Spill &S, int64_t k)
	{
		Mix::Rec r = Mix::from_spill(S, k, g);
		return tile_of(g, r.cell & ((1 << g.lcx) - 1), r.cell >> g.lcx);
	}
};

template <class F>
__global__ void k_rb_count(Grid g, Spill S, int64_t n, int32_t *newcnt)
{
	for(int64_t k = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; k < n;
			k += (int64_t) gridDim.x * blockDim.x)
		atomicAdd(&newcnt[TileOf<F>::get(g, S, k)], 1);
}

// Copy each tile's particles from the old store to the new base: its main
// region, then its pending arrivals (buffer olda.arr_r).
template <class F>
__global__ void k_rb_copy(const PushArgs olda, const PushArgs newa, int s)
{
	const int t = blockIdx.x;
	const Tiles &T = olda.tiles[s];
	const int n = T.cnt[t];
	const int na = min(T.acnt[olda.arr_r][t], T.acap[t]);
	const int64_t ob = T.base[t], nb = newa.tiles[s].base[t];
	const int64_t oab = T.abase[t] + (olda.arr_r ? T.abuf1 : 0);
	for(int i = threadIdx.x; i < n + na; i += blockDim.x)
	{
		typename F::Rec r = F::load(olda, s, i < n ? ob + i : oab + (i - n));
		F::store(newa, s, nb + i, r);
	}
}

// Particles of each tile: its main region's and its pending arrivals.
__global__ void k_tile_total(int nt, const Tiles T, int abuf, int32_t *out)
{
	for(int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x)
		out[t] = T.cnt[t] + min(T.acnt[abuf][t], T.acap[t]);
}

template <class F>
__global__ void k_rb_scatter(const PushArgs newa, int s, Spill S, int64_t n, int32_t *fill)
{
	const Grid &g = newa.g;
	for(int64_t k = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; k < n;
			k += (int64_t) gridDim.x * blockDim.x)
	{
		int t = TileOf<F>::get(g, S, k);
		int slot = atomicAdd(&fill[t], 1);
		typename F::Rec r = F::from_spill(S, k, g);
		F::store(newa, s, newa.tiles[s].base[t] + slot, r);
	}
}

// Tile of a record in the store layout.
template <class F> struct RecTile;
template <> struct RecTile<F64> {
	static __device__ __forceinline__ int get(const Grid &g, const F64::Rec &r)
	{
		double w[4];
		int cx, cy;
		F64::weights(g, r.x, r.y, w, cx, cy);
		cx = min(max(cx, 0), g.nx - 1);
		cy = min(max(cy, 0), g.ny - 1);
		return tile_of(g, cx, cy);
	}
};
template <> struct RecTile<Mix> {
	static __device__ __forceinline__ int get(const Grid &g, const Mix::Rec &r)
	{
		return tile_of(g, r.cell & ((1 << g.lcx) - 1), r.cell >> g.lcx);
	}
};

// Upload, step 1: every staged record converted once to the store's form
// (the FP64 work of the upload, done once), in staging order, into a
// temporary store, with its bucket key (ux >= 0 ? nt : 0) + tile in a key
// column.  Block-local histograms (shared-memory atomics, one global atomic
// per block and bin) give each tile's count and its count of left movers.
// Blocks take contiguous ranges.  Shared memory: 2 nt ints.
template <class F>
__global__ void k_rb_convert(const PushArgs tmp, int s, Spill S, int64_t n, int nt, int32_t *key,
		int32_t *cnt, int32_t *neg)
{
	extern __shared__ int32_t shb[];
	const Grid &g = tmp.g;
	for(int i = threadIdx.x; i < 2 * nt; i += blockDim.x) shb[i] = 0;
	__syncthreads();
	int64_t per = (n + gridDim.x - 1) / gridDim.x;
	int64_t lo = (int64_t) blockIdx.x * per, hi = min(n, lo + per);
	for(int64_t k = lo + threadIdx.x; k < hi; k += blockDim.x)
	{
		typename F::Rec r = F::from_spill(S, k, g);
		const int kk = (r.ux >= 0 ? nt : 0) + RecTile<F>::get(g, r);
		F::store(tmp, s, k, r);
		key[k] = kk;
		atomicAdd(&shb[kk], 1);
	}
	__syncthreads();
	for(int t = threadIdx.x; t < nt; t += blockDim.x)
	{
		int a = shb[t], b = shb[nt + t];
		if(a) atomicAdd(&neg[t], a);
		if(a + b) atomicAdd(&cnt[t], a + b);
	}
}

// Upload, steps 2 and 3: the converted records move to per-bucket runs.
// kRows: buckets are rows of tiles (output grouped by row); else buckets
// are the keys themselves, (direction of ux, tile), so inside every tile
// the particles moving left come first.  Blocks take contiguous ranges of
// the input.  A block numbers the buckets its range can hold locally (all
// rows in pass 1; in pass 2, whose input is grouped by row, the tiles of
// the rows its range spans, in both directions), counts its records per
// bucket from the key column, and reserves one run per bucket at the
// bucket's cursor (one 64-bit global atomic per bucket and block).  Then,
// per batch of kRbBatch records: a shared histogram and scan order the
// batch by bucket in shared memory, and consecutive threads write
// consecutive slots of each run, so the stores coalesce (scattering
// records one by one left the passes 3 to 6 times slower than this).
// A block whose range spans more than kRbMaxLocal buckets (very uneven
// rows) stores record by record at the global cursors instead.
constexpr int kRbThreads = 512;
constexpr int kRbBatch = 2048;
constexpr int kRbMaxLocal = 2048;

template <class F>
constexpr size_t rb_smem_bytes()
{
	return (size_t) kRbMaxLocal * (8 + 4 + 4 + 4)
		+ (size_t) kRbBatch * (4 + 4 + sizeof(typename F::Rec));
}

// Exclusive block-wide scan of v[0, n) into out (n <= 4 kRbThreads); ends
// with a block barrier, so out[] is complete for every thread on return.
__device__ __forceinline__ void rb_scan(const int32_t *v, int32_t *out, int n, int32_t *wsum)
{
	const int t = threadIdx.x, lane = t & 31, w = t >> 5;
	int a[4], sum = 0;
	#pragma unroll
	for(int k = 0; k < 4; k++)
	{
		const int i = 4 * t + k;
		a[k] = i < n ? v[i] : 0;
		sum += a[k];
	}
	int incl = sum;
	for(int o = 1; o < 32; o <<= 1)
	{
		const int y = __shfl_up_sync(0xffffffffu, incl, o);
		if(lane >= o) incl += y;
	}
	if(lane == 31) wsum[w] = incl;
	__syncthreads();
	if(w == 0)
	{
		int x = lane < kRbThreads / 32 ? wsum[lane] : 0;
		int xi = x;
		for(int o = 1; o < 32; o <<= 1)
		{
			const int y = __shfl_up_sync(0xffffffffu, xi, o);
			if(lane >= o) xi += y;
		}
		if(lane < kRbThreads / 32) wsum[lane] = xi - x;
	}
	__syncthreads();
	int run = wsum[w] + incl - sum;
	#pragma unroll
	for(int k = 0; k < 4; k++)
	{
		const int i = 4 * t + k;
		if(i < n) out[i] = run;
		run += a[k];
	}
	// every thread reads out[] of other threads next
	__syncthreads();
}

template <class F, bool kRows>
__global__ void __launch_bounds__(kRbThreads)
k_rb_pass(const PushArgs in, const int32_t *kin, const PushArgs out, int32_t *kout, int s,
		int64_t n, int nrow, unsigned long long *cursor, int64_t ncap_out)
{
	// every index below is in range by construction; the checks only turn
	// a broken invariant into a status bit (ST_RANGE) instead of a stray
	// access
	typedef typename F::Rec Rec;
	extern __shared__ __align__(16) unsigned char shraw[];
	unsigned long long *off = reinterpret_cast<unsigned long long *>(shraw);
	int32_t *run = reinterpret_cast<int32_t *>(off + kRbMaxLocal);
	int32_t *bh = run + kRbMaxLocal;            // batch (or block) counts
	int32_t *bs = bh + kRbMaxLocal;             // batch starts
	int32_t *slb = bs + kRbMaxLocal;            // bucket of each staged slot
	int32_t *skey = slb + kRbBatch;             // key of each staged slot
	Rec *srec = reinterpret_cast<Rec *>(skey + kRbBatch);
	__shared__ int32_t wsum[kRbThreads / 32];
	const Grid &g = out.g;
	const int nt = g.ntx * g.nty;
	const int ntx = g.ntx;
	const int64_t per = (n + gridDim.x - 1) / gridDim.x;
	const int64_t lo = (int64_t) blockIdx.x * per, hi = min(n, lo + per);
	if(lo >= hi) return;
	// the tile of a key, and the row of a tile
	auto key_tile = [&](int key) -> int { return key >= nt ? key - nt : key; };
	auto row_of = [&](int tile) -> int {
		return (int) bits::div_q((uint32_t) tile, g.ntx_mul, g.ntx_sh);
	};
	// local buckets: pass 1 all rows; pass 2 the rows [r0, r0 + R) of
	// this range (its input is grouped by row), left movers first
	const int r0 = kRows ? 0 : row_of(key_tile(kin[lo]));
	const int R = kRows ? nrow : row_of(key_tile(kin[hi - 1])) - r0 + 1;
	const int nbl = kRows ? nrow : 2 * R * ntx;
	auto local = [&](int key) -> int {
		const int tile = key_tile(key);
		if(kRows) return row_of(tile);
		return (key >= nt ? R * ntx : 0) + tile - r0 * ntx;
	};
	auto global = [&](int l) -> int {
		if(kRows) return l;
		const int right = l >= R * ntx;
		return (right ? nt : 0) + r0 * ntx + l - (right ? R * ntx : 0);
	};
	if(nbl > kRbMaxLocal)
	{
		for(int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x)
		{
			const int key = kin[i];
			const int gb = kRows ? row_of(key_tile(key)) : key;
			if(key < 0 || key >= 2 * nt) { set_status(out.status, ST_RANGE); continue; }
			const int64_t dst = (int64_t) atomicAdd(&cursor[gb], 1ULL);
			if(dst < 0 || dst >= ncap_out) { set_status(out.status, ST_RANGE); continue; }
			F::store(out, s, dst, F::load(in, s, i));
			if(kout) kout[dst] = key;
		}
		return;
	}
	for(int l = threadIdx.x; l < nbl; l += blockDim.x) bh[l] = 0;
	__syncthreads();
	for(int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x)
	{
		const int l = local(kin[i]);
		if(l >= 0 && l < nbl) atomicAdd(&bh[l], 1);
		else set_status(out.status, ST_RANGE);
	}
	__syncthreads();
	for(int l = threadIdx.x; l < nbl; l += blockDim.x)
	{
		const int c = bh[l];
		if(c) off[l] = atomicAdd(&cursor[global(l)], (unsigned long long) c);
		run[l] = 0;
		bh[l] = 0;
	}
	__syncthreads();
	constexpr int kPer = kRbBatch / kRbThreads;
	for(int64_t b0 = lo; b0 < hi; b0 += kRbBatch)
	{
		const int m = (int) min((int64_t) kRbBatch, hi - b0);
		int ll[kPer], rk[kPer], ky[kPer];
		#pragma unroll
		for(int k = 0; k < kPer; k++)
		{
			const int j = k * kRbThreads + threadIdx.x;
			ll[k] = -1;
			if(j < m)
			{
				ky[k] = kin[b0 + j];
				const int l = local(ky[k]);
				if(l >= 0 && l < nbl)
				{
					ll[k] = l;
					rk[k] = atomicAdd(&bh[l], 1);
				}
			}
		}
		__syncthreads();
		rb_scan(bh, bs, nbl, wsum);                 // ends with a barrier
		#pragma unroll
		for(int k = 0; k < kPer; k++)
			if(ll[k] >= 0)
			{
				const int pos = bs[ll[k]] + rk[k];
				if(pos < 0 || pos >= kRbBatch) { set_status(out.status, ST_RANGE); continue; }
				slb[pos] = ll[k];
				skey[pos] = ky[k];
				srec[pos] = F::load(in, s, b0 + k * kRbThreads + threadIdx.x);
			}
		__syncthreads();
		// slots in bucket order: consecutive threads, consecutive stores
		// (the batch's valid records fill slots [0, mv))
		const int mv = nbl > 0 ? bs[nbl - 1] + bh[nbl - 1] : 0;
		for(int j = threadIdx.x; j < mv; j += blockDim.x)
		{
			const int l = slb[j];
			if(l < 0 || l >= nbl) { set_status(out.status, ST_RANGE); continue; }
			const int64_t dst = (int64_t) off[l] + run[l] + (j - bs[l]);
			if(dst < 0 || dst >= ncap_out) { set_status(out.status, ST_RANGE); continue; }
			F::store(out, s, dst, srec[j]);
			if(kout) kout[dst] = skey[j];
		}
		__syncthreads();
		for(int l = threadIdx.x; l < nbl; l += blockDim.x)
		{
			run[l] += bh[l];
			bh[l] = 0;
		}
		__syncthreads();
	}
}

// Pass-2 cursors: left movers of tile t from base[t], right movers after
// all of them.
__global__ void k_rb_cursors(int nt, const int64_t *base, const int32_t *neg,
		unsigned long long *cur)
{
	for(int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x)
	{
		cur[t] = (unsigned long long) base[t];
		cur[nt + t] = (unsigned long long) (base[t] + neg[t]);
	}
}

// Upload check, numbering and Y wrap of a staged species.  out[0]: any
// invalid record (x outside [0, Lx], non-finite y, ux, uy); out[1]: the
// largest |ux|, |uy| as the bit pattern of a non-negative double.
__global__ void k_upload_check(int64_t n, Spill S, double Lx, double Ly, unsigned long long *out)
{
	unsigned long long bad = 0;
	double vm = 0.0;
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
			i += (int64_t) gridDim.x * blockDim.x)
	{
		double x = S.x[i], y = S.y[i], u = S.ux[i], v = S.uy[i];
		if(!(x >= 0.0 && x <= Lx) || !isfinite(y) || !isfinite(u) || !isfinite(v))
			bad = 1;
		else
		{
			vm = fmax(vm, fmax(fabs(u), fabs(v)));
			// one periodic wrap in Y, as the initial global exchange does
			// (sim_pre_step -> comm_plasma(sim, 1), comm_plasma.c:1087-1112)
			if(y >= Ly) S.y[i] = y - Ly;
			else if(y < 0.0) S.y[i] = y + Ly;
		}
		S.id[i] = (int32_t) i;
	}
	for(int o = 16; o > 0; o >>= 1)
	{
		bad |= __shfl_xor_sync(0xffffffffu, bad, o);
		vm = fmax(vm, __shfl_xor_sync(0xffffffffu, vm, o));
	}
	if((threadIdx.x & 31) == 0)
	{
		if(bad) atomicOr(&out[0], 1ULL);
		atomicMax(&out[1], (unsigned long long) __double_as_longlong(vm));
	}
}

// Host view: FP64 state by particle id, or (prefix non-null) in store
// order, tile t's particles from prefix[t] on.
template <class F>
__global__ void k_download(const PushArgs a, int s, double *x, double *y, double *ux,
		double *uy, const int64_t *prefix)
{
	int t = blockIdx.x;
	int n = a.tiles[s].cnt[t];
	int64_t b = a.tiles[s].base[t];
	for(int i = threadIdx.x; i < n; i += blockDim.x)
	{
		typename F::Rec r = F::load(a, s, b + i);
		double px, py, pu, pv;
		F::to_spill_vals(r, a.g, px, py, pu, pv);
		int64_t dst = prefix ? prefix[t] + i : (int64_t) r.id;
		x[dst] = px; y[dst] = py; ux[dst] = pu; uy[dst] = pv;
	}
}

template <class F>
__global__ void k_cell_counts(const PushArgs a, int s, unsigned long long *counts)
{
	int t = blockIdx.x;
	int n = a.tiles[s].cnt[t];
	int64_t b = a.tiles[s].base[t];
	for(int i = threadIdx.x; i < n; i += blockDim.x)
	{
		typename F::Rec r = F::load(a, s, b + i);
		int cx, cy;
		F::cell_of(r, a.g, cx, cy);
		if(cx >= 0 && cx < a.g.nx && cy >= 0 && cy < a.g.ny)
			atomicAdd(&counts[(int64_t) cy * a.g.nx + cx], 1ULL);
	}
}

// Per-tile partial sums of m|u|^2 and m u (FP64), deterministic per tile.
template <class F>
__global__ void k_kinetic(const PushArgs a, int s, double m, double *part)
{
	__shared__ double sh[3][256];
	int t = blockIdx.x;
	int n = a.tiles[s].cnt[t];
	int64_t b = a.tiles[s].base[t];
	double k = 0.0, px = 0.0, py = 0.0;
	for(int i = threadIdx.x; i < n; i += blockDim.x)
	{
		typename F::Rec r = F::load(a, s, b + i);
		double x, y, u, v;
		F::to_spill_vals(r, a.g, x, y, u, v);
		k += u * u + v * v;
		px += u;
		py += v;
	}
	sh[0][threadIdx.x] = k; sh[1][threadIdx.x] = px; sh[2][threadIdx.x] = py;
	__syncthreads();
	for(int st = 128; st > 0; st >>= 1)
	{
		if(threadIdx.x < st)
			for(int c = 0; c < 3; c++)
				sh[c][threadIdx.x] += sh[c][threadIdx.x + st];
		__syncthreads();
	}
	if(threadIdx.x == 0)
	{
		part[3 * t + 0] = 0.5 * m * sh[0][0];
		part[3 * t + 1] = m * sh[1][0];
		part[3 * t + 2] = m * sh[2][0];
	}
}

// Field energy partial sums over rows (one block per row), FP64.
__global__ void k_field_energy(Grid g, const double *Ex, const double *Ey, const float2 *E32,
		const long long *rho, double *part)
{
	__shared__ double sh[2][256];
	int iy = blockIdx.x;
	double e = 0.0;
	long long q = 0;
	for(int ix = threadIdx.x; ix < g.nx; ix += blockDim.x)
	{
		int64_t i = (int64_t) iy * g.nx + ix;
		double ex, ey;
		if(E32) { ex = E32[i].x; ey = E32[i].y; }
		else { ex = Ex[i]; ey = Ey[i]; }
		e += ex * ex + ey * ey;
		q += rho[i];
	}
	sh[0][threadIdx.x] = e;
	sh[1][threadIdx.x] = (double) 0;
	__shared__ long long shq[256];
	shq[threadIdx.x] = q;
	__syncthreads();
	for(int st = 128; st > 0; st >>= 1)
	{
		if(threadIdx.x < st)
		{
			sh[0][threadIdx.x] += sh[0][threadIdx.x + st];
			shq[threadIdx.x] += shq[threadIdx.x + st];
		}
		__syncthreads();
	}
	if(threadIdx.x == 0)
	{
		part[2 * iy] = sh[0][0];
		part[2 * iy + 1] = (double) shq[0];
	}
}

// Fixed point -> FP64; rlo (FP64 form) adds the remainder word.
__global__ void k_rho_to_f64(int64_t n, const long long *rho, double qinv, const long long *rlo,
		double qinv_lo, double *out)
{
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
			i += (int64_t) gridDim.x * blockDim.x)
	{
		double v = (double) rho[i] * qinv;
		if(rlo) v += (double) rlo[i] * qinv_lo;
		out[i] = v;
	}
}

// FP64 -> fixed point: high word and (FP64 form) the exact remainder at the
// 2^m finer scale.
__global__ void k_f64_to_rho(int64_t n, const double *in, double qscale, long long *rho,
		double qlo_mul, long long *rlo)
{
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
			i += (int64_t) gridDim.x * blockDim.x)
	{
		double v = in[i] * qscale;
		long long hi = __double2ll_rn(v);
		rho[i] = hi;
		if(rlo) rlo[i] = __double2ll_rn((v - (double) hi) * qlo_mul);
	}
}

__global__ void k_iota(int64_t n, int32_t *id)
{
	for(int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
			i += (int64_t) gridDim.x * blockDim.x)
		id[i] = (int32_t) i;
}

// ------------------------------------------------------------- helpers

static int grid_blocks(int64_t n, int threads = 256, int maxb = 4096)
{
	int64_t b = (n + threads - 1) / threads;
	if(b < 1) b = 1;
	if(b > maxb) b = maxb;
	return (int) b;
}

static int ilog2(int64_t v)
{
	int l = 0;
	while(((int64_t) 1 << l) < v) l++;
	return l;
}

static bool pow2(int64_t v) { return v > 0 && (v & (v - 1)) == 0; }

static PushArgs make_args(cpic_ctx *c, int cur_spill)
{
	PushArgs a;
	memset(&a, 0, sizeof(a));
	a.g = c->g;
	a.nspecies = c->nspecies;
	a.arr_r = c->spill_cur;
	for(int s = 0; s < c->nspecies; s++)
	{
		a.tiles[s] = c->sp[s].tiles;
		a.f64[s] = c->sp[s].f64;
		a.mix[s] = c->sp[s].mix;
		a.spill_out[s] = c->sp[s].spill[cur_spill ^ 1];
	}
	a.rho = c->rho;
	a.rho_lo = c->rho_lo;
	a.Ex64 = c->Ex64;
	a.Ey64 = c->Ey64;
	a.E32 = c->precision == CPIC_MIXED ? c->E32 : nullptr;
	a.status = c->status;
	if(c->emap_ok)
	{
		a.emap = c->emap;
		a.emap_ok = 1;
	}
	return a;
}

// The mixed form's field tiles as 2D tensor copies: a map of E32 (nx x ny
// elements of 8 bytes, row pitch nx * 8) with a box of (tx + 2) x (ty + 1)
// elements, the tile's (tx + 1) x (ty + 1) nodes padded to an even width.
// The copy engine wants the box's row and its first column on 16-byte
// boundaries (tx even: tile origins and the box width are even), the row
// pitch a multiple of 16 bytes (nx even), at most 256 elements per box
// side and a 128-byte aligned destination (every staged chunk size is a
// multiple of 128 bytes).  Otherwise, or without the driver's encoder,
// the fused kernel loads field tiles by threads.
static bool encode_field_map(cpic_ctx *c)
{
	const Grid &g = c->g;
	if(c->precision != CPIC_MIXED || g.tx % 2 || g.nx % 2 || g.tx + 2 > 256 || g.ty + 1 > 256)
		return false;
	for(int P : kPPTChoices)
		for(int ids = 0; ids < 2; ids++)
			if(Mix::stage_bytes(ids != 0, chunk_of(P)) % 128)
				return false;
	static PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
		void *fn = nullptr;
		cudaDriverEntryPointQueryResult q;
		if(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
				&q) != cudaSuccess || q != cudaDriverEntryPointSuccess)
			fn = nullptr;
		return (PFN_cuTensorMapEncodeTiled_v12000) fn;
	}();
	if(!encode)
		return false;
	const cuuint64_t dims[2] = {(cuuint64_t) g.nx, (cuuint64_t) g.ny};
	const cuuint64_t pitch[1] = {(cuuint64_t) g.nx * sizeof(float2)};
	const cuuint32_t box[2] = {(cuuint32_t) (g.tx + 2), (cuuint32_t) (g.ty + 1)};
	const cuuint32_t step[2] = {1, 1};
	return encode(&c->emap, CU_TENSOR_MAP_DATA_TYPE_INT64, 2, c->E32, dims, pitch, box, step,
			CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
			CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static void fill_species_step(cpic_ctx *c, PushArgs &a, int64_t iter)
{
	const cpic_params_t &p = c->p;
	double dt = iter == 0 ? -p.dt / 2 : p.dt;
	a.iter = (int) (iter == 0 ? 0 : 1);
	a.dt = dt;
	a.cdx_f = (float) (p.dt / c->g.dx);
	a.cdy_f = (float) (p.dt / c->g.dy);
	int64_t chunks = p.plasma_chunks > 0 ? p.plasma_chunks : 1;
	for(int s = 0; s < c->nspecies; s++)
	{
		SpeciesStep &st = a.sp[s];
		double q = c->sp[s].q, m = c->sp[s].m;
		// chunk_update_r, mover.c:204-225
		st.dtqm2 = 0.5 * dt * q / m;
		// boris_rotation, mover.c:43-51
		st.tz = p.B[2] * st.dtqm2;
		double sd = 1.0;
		sd += st.tz * st.tz;
		st.sz = 2.0 * st.tz / sd;
		// umax, sim.c:198-200
		st.umax_x = (c->g.nx / chunks) * c->g.dx / p.dt;
		st.umax_y = c->g.ny * c->g.dy / p.dt;
		double vq = -q / p.e0;
		st.qfix = vq * c->qscale;
		st.qlo_mul = c->qlo_mul;
		st.qlo_exp = ilogb(c->qlo_mul);
		st.wq_scale = c->wq_exact ? c->sp[s].wq_mult : st.qfix * ldexp(1.0, -kWeightBits);
		st.wq_int = c->wq_exact ? (long long) c->sp[s].wq_mult : 0;
		st.dtqm2_f = (float) st.dtqm2;
		st.tz_f = (float) st.tz;
		st.sz_f = (float) st.sz;
		st.umax_x_f = (float) st.umax_x;
		st.umax_y_f = (float) st.umax_y;
	}
}

static size_t push_smem_h(const cpic_ctx *c, int halo)
{
	// two staged chunks plus the form's accumulators and field tile
	int W = c->g.tx + 2 * halo + 1;
	// (+128: the kernel rounds the dynamic base up to 128 bytes)
	const int C = chunk_of(c->ppt);
	if(c->precision == CPIC_MIXED)
		return 128 + 2 * Mix::stage_bytes(c->p.track_ids != 0, C) + Mix::smem_bytes(W, c->g.tx);
	return 128 + 2 * F64::stage_bytes(true, C) + F64::smem_bytes(W, c->g.tx);
}

static size_t push_smem(const cpic_ctx *c)
{
	return push_smem_h(c, c->g.halo);
}

static int check_status(cpic_ctx *c)
{
	uint32_t st = 0;
	CK(cudaStreamSynchronize(c->stream));
	CK(cudaMemcpy(&st, c->status, sizeof(st), cudaMemcpyDeviceToHost));
	if(st & ST_SPILL_FULL) return CPIC_ECAPACITY;
	if(st & ST_UMAX) return CPIC_EUMAX;
	if(st & ST_NAN) return CPIC_ENAN;
	if(st & ST_RANGE) return CPIC_EINVAL;
	if(st & ST_TIMEOUT) return CPIC_ETIMEOUT;
	return CPIC_OK;
}

static int alloc_store(cpic_ctx *c, SpeciesHost &S, int64_t cap, bool alt)
{
	// 16 spare records: no bulk copy rounded up to 16 bytes can reach past
	// the allocation, whatever the last tile's count
	const int64_t nal = cap + 16;
	if(c->precision == CPIC_FP64)
	{
		StoreF64 &st = alt ? S.f64_alt : S.f64;
		CK(cudaMalloc(&st.x, nal * sizeof(double)));
		CK(cudaMalloc(&st.y, nal * sizeof(double)));
		CK(cudaMalloc(&st.ux, nal * sizeof(double)));
		CK(cudaMalloc(&st.uy, nal * sizeof(double)));
		CK(cudaMalloc(&st.id, nal * sizeof(int32_t)));
	}
	else
	{
		StoreMix &st = alt ? S.mix_alt : S.mix;
		CK(cudaMalloc(&st.cell, nal * sizeof(int32_t)));
		CK(cudaMalloc(&st.ou, nal * sizeof(float4)));
		st.id = nullptr;
		if(c->p.track_ids)
			CK(cudaMalloc(&st.id, nal * sizeof(int32_t)));
	}
	return CPIC_OK;
}

static void free_store(cpic_ctx *c, SpeciesHost &S, bool alt)
{
	if(c->precision == CPIC_FP64)
	{
		StoreF64 &st = alt ? S.f64_alt : S.f64;
		cudaFree(st.x); cudaFree(st.y); cudaFree(st.ux); cudaFree(st.uy); cudaFree(st.id);
		memset(&st, 0, sizeof(st));
	}
	else
	{
		StoreMix &st = alt ? S.mix_alt : S.mix;
		cudaFree(st.cell); cudaFree(st.ou);
		cudaFree(st.id);
		memset(&st, 0, sizeof(st));
	}
}

// The count is cleared on the caller's stream, ahead of the work it
// queues there (the context's streams do not synchronise with the legacy
// default stream).
static int alloc_spill(Spill &S, int32_t capacity, cudaStream_t st, int cell_units = 0)
{
	S.capacity = capacity;
	S.cell_units = cell_units;
	CK(cudaMalloc(&S.x, (size_t) capacity * sizeof(double)));
	CK(cudaMalloc(&S.y, (size_t) capacity * sizeof(double)));
	CK(cudaMalloc(&S.ux, (size_t) capacity * sizeof(double)));
	CK(cudaMalloc(&S.uy, (size_t) capacity * sizeof(double)));
	CK(cudaMalloc(&S.id, (size_t) capacity * sizeof(int32_t)));
	CK(cudaMalloc(&S.count, sizeof(int32_t)));
	CK(cudaMemsetAsync(S.count, 0, sizeof(int32_t), st));
	return CPIC_OK;
}

static void free_spill(Spill &S)
{
	cudaFree(S.x); cudaFree(S.y); cudaFree(S.ux); cudaFree(S.uy); cudaFree(S.id);
	cudaFree(S.count);
	memset(&S, 0, sizeof(S));
}

template <class F>
static void launch_rb_copy(const PushArgs &o, const PushArgs &n, int s, int nt, cudaStream_t st)
{
	k_rb_copy<F><<<nt, 256, 0, st>>>(o, n, s);
}

template <class F>
static void launch_rb_scatter(const PushArgs &n, int s, const Spill &S, int64_t cnt,
		int32_t *fill, cudaStream_t st)
{
	if(cnt > 0)
		k_rb_scatter<F><<<grid_blocks(cnt), 256, 0, st>>>(n, s, S, cnt, fill);
}

template <class F>
static void launch_rb_count(const Grid &g, const Spill &S, int64_t cnt, int32_t *newcnt,
		cudaStream_t st)
{
	if(cnt > 0)
		k_rb_count<F><<<grid_blocks(cnt), 256, 0, st>>>(g, S, cnt, newcnt);
}

// Largest tile count of the block-local upload sort (its scatter keeps
// 4 ints per tile in shared memory: 128 KB).
constexpr int kBlkSortMaxTiles = 8192;

// Counting-sort rebuild of species s: its tiles (unless `fresh`), its
// current spill input and an optional staging list are merged into a new
// layout whose tile capacities follow the new counts.
static int rebuild_species(cpic_ctx *c, int s, bool fresh, const Spill *staging, int64_t nstage)
{
	SpeciesHost &S = c->sp[s];
	int nt = c->ntiles;
	cudaStream_t st = c->stream;
	Spill &spin = S.spill[c->spill_cur];
	int32_t nspill = 0;
	CK(cudaMemcpyAsync(&nspill, spin.count, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	if(nspill > spin.capacity) nspill = spin.capacity;

	int32_t *newcnt = nullptr, *fill = nullptr, *negcnt = nullptr;
	CK(cudaMalloc(&newcnt, nt * sizeof(int32_t)));
	CK(cudaMalloc(&fill, nt * sizeof(int32_t)));
	if(fresh)
		CK(cudaMemsetAsync(newcnt, 0, nt * sizeof(int32_t), st));
	else
		k_tile_total<<<grid_blocks(nt), 256, 0, st>>>(nt, S.tiles, c->spill_cur, newcnt);
	bool mix = c->precision == CPIC_MIXED;
	// the upload of a species: one conversion pass (records, keys and the
	// histogram of (tile, sign of ux)), then two sorting passes below
	const bool blk = fresh && staging && nspill == 0 && nstage > 0 && nt <= kBlkSortMaxTiles;
	const int blk_blocks = (int) std::min<int64_t>(152 * 8, (nstage + 4095) / 4096);
	SpeciesHost tmp1, tmp2;
	memset((void *) &tmp1, 0, sizeof(tmp1));
	memset((void *) &tmp2, 0, sizeof(tmp2));
	int32_t *key1 = nullptr, *key2 = nullptr;
	if(blk)
	{
		static PerDeviceOnce once;
		CK(once.run([] {
			return set_max_dyn_smem({(const void *) k_rb_convert<Mix>, (const void *) k_rb_convert<F64>},
					2 * kBlkSortMaxTiles * (int) sizeof(int32_t));
		}));
		int r = alloc_store(c, tmp1, nstage, false);
		if(r) return r;
		CK(cudaMalloc(&key1, nstage * sizeof(int32_t)));
		PushArgs t1 = make_args(c, c->spill_cur);
		t1.f64[s] = tmp1.f64;
		t1.mix[s] = tmp1.mix;
		CK(cudaMalloc(&negcnt, nt * sizeof(int32_t)));
		CK(cudaMemsetAsync(negcnt, 0, nt * sizeof(int32_t), st));
		if(mix)
			k_rb_convert<Mix><<<blk_blocks, 512, 2 * nt * sizeof(int32_t), st>>>(t1, s, *staging,
					nstage, nt, key1, newcnt, negcnt);
		else
			k_rb_convert<F64><<<blk_blocks, 512, 2 * nt * sizeof(int32_t), st>>>(t1, s, *staging,
					nstage, nt, key1, newcnt, negcnt);
		CK(cudaGetLastError());
	}
	else if(mix)
	{
		launch_rb_count<Mix>(c->g, spin, nspill, newcnt, st);
		if(staging) launch_rb_count<Mix>(c->g, *staging, nstage, newcnt, st);
	}
	else
	{
		launch_rb_count<F64>(c->g, spin, nspill, newcnt, st);
		if(staging) launch_rb_count<F64>(c->g, *staging, nstage, newcnt, st);
	}
	std::vector<int32_t> hc(nt);
	CK(cudaMemcpyAsync(hc.data(), newcnt, nt * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));

	// capacities: slack_pct % slack (25 % at first, doubled after every
	// rebuild forced by an overflow, up to 200 %) plus 64 slots, rounded
	// to 32
	// arrivals regions: two buffers after the main regions, each tile
	// with room for a quarter of its count (a step moves about a tenth of
	// the particles of the two-stream workload between tiles), more as
	// overflows raise the slack (a quarter of it in each buffer, so that a
	// store at 200 % slack holds 4x its particles: two such stores, the
	// current one and the alternate, of both forms fit in HBM at 2048^2)
	std::vector<int64_t> hb(nt), hab(nt);
	std::vector<int32_t> hcap(nt), hacap(nt);
	int64_t total = 0, atotal = 0, n = 0;
	const int arr_pct = std::max(25, c->slack_pct / 4);
	for(int t = 0; t < nt; t++)
	{
		int64_t cap = hc[t] + hc[t] * c->slack_pct / 100 + 64;
		cap = (cap + 31) & ~(int64_t) 31;
		int64_t acap = hc[t] * arr_pct / 100 + 64;
		acap = (acap + 31) & ~(int64_t) 31;
		if(cap > INT32_MAX || acap > INT32_MAX) return CPIC_ECAPACITY;
		hb[t] = total;
		hcap[t] = (int32_t) cap;
		hab[t] = atotal;
		hacap[t] = (int32_t) acap;
		total += cap;
		atotal += acap;
		n += hc[t];
	}
	for(int t = 0; t < nt; t++) hab[t] += total;
	const int64_t slots = total + 2 * atotal;

	// the alternate store receives the new layout
	bool have_alt = mix ? S.mix_alt.ou != nullptr : S.f64_alt.ux != nullptr;
	if(S.cap_alt < slots || !have_alt)
	{
		free_store(c, S, true);
		int r = alloc_store(c, S, slots, true);
		if(r) return r;
		S.cap_alt = slots;
	}
	int64_t *nbase;
	int32_t *ncap;
	CK(cudaMalloc(&nbase, nt * sizeof(int64_t)));
	CK(cudaMalloc(&ncap, nt * sizeof(int32_t)));
	CK(cudaMemcpyAsync(nbase, hb.data(), nt * sizeof(int64_t), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(ncap, hcap.data(), nt * sizeof(int32_t), cudaMemcpyHostToDevice, st));

	PushArgs olda = make_args(c, c->spill_cur);
	PushArgs newa = olda;
	newa.tiles[s].base = nbase;
	newa.tiles[s].cap = ncap;
	newa.f64[s] = S.f64_alt;
	newa.mix[s] = S.mix_alt;
	// the spill records go after each tile's copied particles
	if(fresh)
		CK(cudaMemsetAsync(fill, 0, nt * sizeof(int32_t), st));
	else
		k_tile_total<<<grid_blocks(nt), 256, 0, st>>>(nt, S.tiles, c->spill_cur, fill);
	if(!fresh)
	{
		if(mix) launch_rb_copy<Mix>(olda, newa, s, nt, st);
		else launch_rb_copy<F64>(olda, newa, s, nt, st);
	}
	if(blk)
	{
		// pass 1: by row of tiles into a temporary store; pass 2: by
		// (direction, tile) into the new layout
		const int ntx = c->g.ntx;                      // tiles per row
		const int nrow = c->g.nty;
		std::vector<unsigned long long> rowcur(nrow);
		unsigned long long acc = 0;
		for(int r = 0; r < nrow; r++)
		{
			rowcur[r] = acc;
			for(int t = r * ntx; t < (r + 1) * ntx; t++) acc += (unsigned long long) hc[t];
		}
		int r = alloc_store(c, tmp2, nstage, false);
		if(r) return r;
		CK(cudaMalloc(&key2, nstage * sizeof(int32_t)));
		PushArgs t1 = newa, t2 = newa;
		t1.f64[s] = tmp1.f64;
		t1.mix[s] = tmp1.mix;
		t2.f64[s] = tmp2.f64;
		t2.mix[s] = tmp2.mix;
		unsigned long long *cur = nullptr;
		CK(cudaMalloc(&cur, std::max(nrow, 2 * nt) * sizeof(unsigned long long)));
		CK(cudaMemcpyAsync(cur, rowcur.data(), nrow * sizeof(unsigned long long),
				cudaMemcpyHostToDevice, st));
		static PerDeviceOnce pass_once;
		CK(pass_once.run([] {
			const int mm = (int) rb_smem_bytes<Mix>(), mf = (int) rb_smem_bytes<F64>();
			cudaError_t e = set_max_dyn_smem({(const void *) k_rb_pass<Mix, true>,
					(const void *) k_rb_pass<Mix, false>}, mm);
			return e != cudaSuccess ? e : set_max_dyn_smem({(const void *) k_rb_pass<F64, true>,
					(const void *) k_rb_pass<F64, false>}, mf);
		}));
		const int pb = 152 * 2;
		const size_t smm = rb_smem_bytes<Mix>(), smf = rb_smem_bytes<F64>();
		if(mix)
			k_rb_pass<Mix, true><<<pb, kRbThreads, smm, st>>>(t1, key1, t2, key2, s, nstage, nrow, cur,
					nstage);
		else
			k_rb_pass<F64, true><<<pb, kRbThreads, smf, st>>>(t1, key1, t2, key2, s, nstage, nrow, cur,
					nstage);
		CK(cudaGetLastError());
		k_rb_cursors<<<(nt + 255) / 256, 256, 0, st>>>(nt, nbase, negcnt, cur);
		if(mix)
			k_rb_pass<Mix, false><<<pb, kRbThreads, smm, st>>>(t2, key2, newa, nullptr, s, nstage,
					nrow, cur, total);
		else
			k_rb_pass<F64, false><<<pb, kRbThreads, smf, st>>>(t2, key2, newa, nullptr, s, nstage,
					nrow, cur, total);
		CK(cudaGetLastError());
		CK(cudaStreamSynchronize(st));
		cudaFree(cur);
		cudaFree(key1);
		cudaFree(key2);
		free_store(c, tmp1, false);
		free_store(c, tmp2, false);
		cudaFree(negcnt);
	}
	else if(mix)
	{
		launch_rb_scatter<Mix>(newa, s, spin, nspill, fill, st);
		if(staging) launch_rb_scatter<Mix>(newa, s, *staging, nstage, fill, st);
	}
	else
	{
		launch_rb_scatter<F64>(newa, s, spin, nspill, fill, st);
		if(staging) launch_rb_scatter<F64>(newa, s, *staging, nstage, fill, st);
	}
	CK(cudaGetLastError());
	CK(cudaMemsetAsync(spin.count, 0, sizeof(int32_t), st));
	CK(cudaMemcpyAsync(S.tiles.cnt, newcnt, nt * sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
	CK(cudaMemcpyAsync(S.tiles.base, nbase, nt * sizeof(int64_t), cudaMemcpyDeviceToDevice, st));
	CK(cudaMemcpyAsync(S.tiles.cap, ncap, nt * sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
	CK(cudaMemcpyAsync(S.tiles.abase, hab.data(), nt * sizeof(int64_t), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(S.tiles.acap, hacap.data(), nt * sizeof(int32_t), cudaMemcpyHostToDevice, st));
	CK(cudaMemsetAsync(S.tiles.acnt[0], 0, nt * sizeof(int32_t), st));
	CK(cudaMemsetAsync(S.tiles.acnt[1], 0, nt * sizeof(int32_t), st));
	S.tiles.abuf1 = atotal;
	CK(cudaStreamSynchronize(st));
	cudaFree(nbase); cudaFree(ncap); cudaFree(newcnt); cudaFree(fill);
	// swap stores; the old one becomes the alternate
	std::swap(S.f64, S.f64_alt);
	std::swap(S.mix, S.mix_alt);
	std::swap(S.cap_main, S.cap_alt);
	S.n = n;
	return CPIC_OK;
}

// Every species' pending arrivals (buffer spill_cur) into the main regions
// where they fit; returns in *unmerged the number of tiles where they did
// not (synchronises the context's stream).
static int merge_arrivals(cpic_ctx *c, int32_t *unmerged)
{
	*unmerged = 0;
	if(c->nspecies == 0) return CPIC_OK;
	PushArgs a = make_args(c, c->spill_cur);
	CK(cudaMemsetAsync(c->counter, 0, sizeof(int32_t), c->stream));
	dim3 grid(c->ntiles, c->nspecies);
	if(c->precision == CPIC_MIXED)
		k_merge<Mix><<<grid, 256, 0, c->stream>>>(a, c->counter);
	else
		k_merge<F64><<<grid, 256, 0, c->stream>>>(a, c->counter);
	CK(cudaGetLastError());
	CK(cudaMemcpyAsync(unmerged, c->counter, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return CPIC_OK;
}

// Records in a species' spill list above which a step rebuilds the layout.
// The spill pass pushes the records every step (about as fast as the fused
// kernel per particle, but with global atomics), while a rebuild of the
// two-stream 2048x2048 store takes ~7 ms; rebuilding at the first spilled
// record rebuilt 71 times over that workload's bunching with a check after
// every step (0.67 s of its 4.0 s).
static int32_t spill_threshold(const cpic_ctx *c, int s)
{
	const SpeciesHost &S = c->sp[s];
	int64_t t = std::max<int64_t>(4096, S.n / 1024);
	return (int32_t) std::min<int64_t>(t, S.spill[0].capacity / 4);
}

// After the context's stream has been synchronised: rebuilds the layout of
// every species whose spill list holds records (all: any record; else more
// than spill_threshold), a rebuild taking the main regions, the pending
// arrivals and the spill list.  *rebuilt (optional) says whether one ran.
static int rebuild_if_spilled(cpic_ctx *c, bool all = true, bool *rebuilt = nullptr)
{
	c->last_spill = 0;
	if(rebuilt) *rebuilt = false;
	for(int s = 0; s < c->nspecies; s++)
	{
		int32_t ns = 0;
		CK(cudaMemcpy(&ns, c->sp[s].spill[c->spill_cur].count, sizeof(int32_t),
				cudaMemcpyDeviceToHost));
		c->last_spill += ns;
		if(ns > (all ? 0 : spill_threshold(c, s)))
		{
			// a tile overflowed: more headroom from now on
			c->rebuilds++;
			c->slack_pct = std::min(200, 2 * c->slack_pct);
			int r = rebuild_species(c, s, false, nullptr, 0);
			if(r) return r;
			if(rebuilt) *rebuilt = true;
		}
	}
	return CPIC_OK;
}

// After a particle stage: the status word and the spill counts in one round
// trip (pinned host copies, one synchronisation); a rebuild only when a
// spill list has grown past its threshold.
static int step_check(cpic_ctx *c)
{
	cudaStream_t st = c->stream;
	CK(cudaMemcpyAsync(&c->probe_h[0], c->status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
	for(int s = 0; s < c->nspecies; s++)
		CK(cudaMemcpyAsync(&c->probe_h[1 + s], c->sp[s].spill[c->spill_cur].count,
				sizeof(int32_t), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	const uint32_t sw = (uint32_t) c->probe_h[0];
	if(sw & ST_SPILL_FULL) return CPIC_ECAPACITY;
	if(sw & ST_UMAX) return CPIC_EUMAX;
	if(sw & ST_NAN) return CPIC_ENAN;
	if(sw & ST_RANGE) return CPIC_EINVAL;
	if(sw & ST_TIMEOUT) return CPIC_ETIMEOUT;
	bool over = false;
	c->last_spill = 0;
	for(int s = 0; s < c->nspecies; s++)
	{
		c->last_spill += c->probe_h[1 + s];
		over = over || c->probe_h[1 + s] > spill_threshold(c, s);
	}
	return over ? rebuild_if_spilled(c, false) : CPIC_OK;
}

// Whether ordering the tiles can shorten the fused kernel: only when its
// blocks do not all fit on the GPU at once (more than one wave), and the
// layout is small enough for the one-block sort.
static bool tile_order_pays(const cpic_ctx *c, size_t smem)
{
	if(c->ntiles > kOrderMaxTiles)
		return false;
	int dev = 0, nsm = 0;
	if(cudaGetDevice(&dev) != cudaSuccess
			|| cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
		return true;
	const int per_sm = c->precision == CPIC_MIXED
		? push_mix_blocks_per_sm(smem, c->p.track_ids != 0, c->ppt, c->g.pow2 != 0)
		: push_f64_blocks_per_sm(smem, c->ppt);
	return per_sm <= 0 || (int64_t) c->ntiles > (int64_t) per_sm * nsm;
}

// One fused particle stage (gather, push, re-bin, deposit) without
// host synchronisation.  deposit_only: the initial charge deposit.
static int plasma_stage_async(cpic_ctx *c, bool deposit_only, cudaEvent_t ev0 = nullptr,
		cudaEvent_t ev1 = nullptr)
{
	cudaStream_t st = c->stream;
	int64_t ng = (int64_t) c->g.nx * c->g.ny;
	CK(cudaMemsetAsync(c->rho, 0, ng * sizeof(long long), st));
	if(c->rho_lo)
		CK(cudaMemsetAsync(c->rho_lo, 0, ng * sizeof(long long), st));
	int cur = c->spill_cur;
	for(int s = 0; s < c->nspecies; s++)
		CK(cudaMemsetAsync(c->sp[s].spill[cur ^ 1].count, 0, sizeof(int32_t), st));
	SpillArgs sa;
	memset(&sa, 0, sizeof(sa));
	sa.p = make_args(c, cur);
	fill_species_step(c, sa.p, deposit_only ? 0 : c->iter);
	if(deposit_only)
	{
		// no field, no push: deposit the current positions (pre-step)
		for(int s = 0; s < c->nspecies; s++)
		{
			sa.p.sp[s].dtqm2 = 0.0; sa.p.sp[s].tz = 0.0; sa.p.sp[s].sz = 0.0;
			sa.p.sp[s].dtqm2_f = 0.0f; sa.p.sp[s].tz_f = 0.0f; sa.p.sp[s].sz_f = 0.0f;
			sa.p.sp[s].umax_x = INFINITY; sa.p.sp[s].umax_y = INFINITY;
			sa.p.sp[s].umax_x_f = INFINITY; sa.p.sp[s].umax_y_f = INFINITY;
		}
		sa.p.iter = 0;
	}
	for(int s = 0; s < c->nspecies; s++)
		sa.spill_in[s] = c->sp[s].spill[cur];
	size_t smem = push_smem(c);
	// the spill pass first: its records go to their tiles or to the empty
	// output list (same capacity as its input), so none can be lost; the
	// fused kernel's own overflow then falls back to staying in its tile
	if(c->precision == CPIC_MIXED)
		launch_spill_mix(sa, st);
	else
		launch_spill_f64(sa, st);
	if(ev0) CK(cudaEventRecord(ev0, st));
	if(c->precision == CPIC_MIXED)
		CK(launch_push_mix(sa.p, c->ntiles, smem, c->ppt, st));
	else
		CK(launch_push_f64(sa.p, c->ntiles, smem, c->ppt, st));
	if(ev1) CK(cudaEventRecord(ev1, st));
	CK(cudaGetLastError());
	// the next launch's tile order, from the main regions' counts and the
	// arrivals this launch left for it
	if(c->order_mode == 0)
		c->order_mode = tile_order_pays(c, smem) ? 1 : 2;
	if(c->order_mode == 1)
		k_tile_order<<<c->nspecies, kOrderThreads, 0, st>>>(sa.p, c->ntiles, cur ^ 1);
	CK(cudaGetLastError());
	c->spill_cur ^= 1;
	return CPIC_OK;
}

// The state host reads and re-layouts walk: every particle in a main region
// (arrivals merged, the spill list rebuilt into the tiles if anything
// overflowed).
static int normalize(cpic_ctx *c)
{
	CK(cudaStreamSynchronize(c->stream));
	int r = rebuild_if_spilled(c);
	if(r) return r;
	int32_t unmerged = 0;
	if((r = merge_arrivals(c, &unmerged))) return r;
	// arrivals that did not fit their tile's main region: a new layout
	// (the main regions full: more headroom from now on)
	if(unmerged > 0)
	{
		c->rebuilds++;
		c->slack_pct = std::min(200, 2 * c->slack_pct);
		for(int s = 0; s < c->nspecies; s++)
			if((r = rebuild_species(c, s, false, nullptr, 0))) return r;
	}
	return CPIC_OK;
}

static int field_stage_async(cpic_ctx *c)
{
	cudaStream_t st = c->stream;
	if(c->precision == CPIC_MIXED)
	{
		// the mean charge density the particles carry (each deposits
		// -q/e0 in all, sum_s n_s (-q_s/e0) over the nx ny nodes): removed
		// before the FP32 transform
		double tot = 0.0;
		for(int s = 0; s < c->nspecies; s++)
			tot += (double) c->sp[s].n * (-c->sp[s].q / c->p.e0);
		double mean0 = tot / ((double) c->g.nx * (double) c->g.ny);
		CK(launch_poisson_mix(c->g, c->rho, c->qinv, nullptr, c->spec32, c->twx32, c->twy32,
				c->cosx, c->cosy, c->phi32, st, c->green32, mean0));
		launch_E_mix(c->g, c->phi32, c->E32, st);
	}
	else
	{
		CK(launch_poisson_f64(c->g, c->rho, c->qinv, c->spec64, c->twx64, c->twy64,
				c->cosx, c->cosy, c->phi64, st, c->rho_lo, c->qinv_lo, c->green64));
		launch_E_f64(c->g, c->phi64, c->Ex64, c->Ey64, st);
	}
	CK(cudaGetLastError());
	return CPIC_OK;
}

static int ensure_scratch(cpic_ctx *c, size_t n)
{
	if(c->scratch_n >= n) return CPIC_OK;
	cudaFree(c->scratch);
	c->scratch = nullptr;
	CK(cudaMalloc(&c->scratch, n * sizeof(double)));
	c->scratch_n = n;
	return CPIC_OK;
}

// ------------------------------------------------------------- C ABI

extern "C" {

CPIC_API int cpic_create(const cpic_params_t *p, cpic_ctx_t **out)
{
	if(!p || !out) return CPIC_EINVAL;
	*out = nullptr;
	// any grid from 4 x 4 to 16384 x 16384 cells (the reference's FFTW
	// solver takes any nx, ny: solver.c:246-330)
	if(p->nx < 4 || p->ny < 4 || p->nx > (1 << 14) || p->ny > (1 << 14))
		return CPIC_EINVAL;
	if(!(p->Lx > 0) || !(p->Ly > 0) || !(p->dt > 0) || !(p->e0 > 0))
		return CPIC_EINVAL;
	// The reference rejects any non-zero u_z (umax[Z] = 0, mover.c:97-137,
	// sim.c:200), which an in-plane B would produce on the first step.
	if(p->B[0] != 0.0 || p->B[1] != 0.0)
		return CPIC_EINVAL;
	if(p->precision != CPIC_FP64 && p->precision != CPIC_MIXED)
		return CPIC_EINVAL;
	int ndev = 0;
	if(cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
		return CPIC_ENODEV;

	cpic_ctx *c = new cpic_ctx();
	memset((void *) c, 0, sizeof(*c));
	c->slack_pct = 25;
	c->p = *p;
	c->precision = p->precision;
	c->iter = -1;
	Grid &g = c->g;
	g.nx = (int) p->nx; g.ny = (int) p->ny;
	g.Lx = p->Lx; g.Ly = p->Ly;
	// sim_prepare, sim.c:171-175
	g.dx = p->Lx / p->nx;
	g.dy = p->Ly / p->ny;
	// interpolate_f2p_E / interpolate_p2f_rho, interpolate.c:303-304
	g.idx = 1.0 / g.dx;
	g.idy = 1.0 / g.dy;
	int T = p->tile_x;
	if(T <= 0)
	{
		// default: the largest tile with at least 2048 tiles, else the
		// largest tile giving at least 64 tiles, else the largest power of
		// two up to 32 dividing both sides (1 for an odd side)
		T = 0;
		for(int cand = 64; cand >= 4 && !T; cand >>= 1)
			if(p->nx % cand == 0 && p->ny % cand == 0
					&& (p->nx / cand) * (p->ny / cand) >= 2048) T = cand;
		for(int cand = 32; cand >= 4 && !T; cand >>= 1)
			if(p->nx % cand == 0 && p->ny % cand == 0
					&& (p->nx / cand) * (p->ny / cand) >= 64) T = cand;
		for(int cand = 32; cand >= 1 && !T; cand >>= 1)
			if(p->nx % cand == 0 && p->ny % cand == 0) T = cand;
	}
	int TY = p->tile_y > 0 ? p->tile_y : T;
	if(!pow2(T) || !pow2(TY) || p->nx % T || p->ny % TY || T != TY)
	{
		delete c;
		return CPIC_EINVAL;
	}
	c->ppt = p->particles_per_thread > 0 ? p->particles_per_thread : kPPT;
	if(!ppt_supported(c->ppt))
	{
		delete c;
		return CPIC_EINVAL;
	}
	g.tx = T; g.ty = TY;
	g.ntx = g.nx / T; g.nty = g.ny / TY;
	g.halo = p->halo > 0 ? p->halo : 2;
	g.lcx = ilog2(g.nx);
	g.ltx = ilog2(T); g.lty = ilog2(TY);
	bits::div_init((uint32_t) g.ntx, g.ntx_mul, g.ntx_sh);
	g.pow2 = pow2(g.nx) && pow2(g.ny);
	c->ntiles = g.ntx * g.nty;
	if(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
	{
		delete c;
		return CPIC_ECUDA;
	}
	if(cudaMallocHost((void **) &c->probe_h, (1 + kMaxSpecies) * sizeof(int32_t)) != cudaSuccess)
	{
		cudaStreamDestroy(c->stream);
		delete c;
		return CPIC_ENOMEM;
	}
	int64_t ng = (int64_t) g.nx * g.ny;
	int64_t nh = g.nx / 2 + 1;
	int r = CPIC_OK;
#define AL(ptr, bytes) do { if(cudaMalloc(&(ptr), (bytes)) != cudaSuccess) { r = CPIC_ENOMEM; goto fail; } } while(0)
	AL(c->rho, ng * sizeof(long long));
	AL(c->status, sizeof(uint32_t));
	AL(c->cosx, g.nx * sizeof(double));
	AL(c->cosy, g.ny * sizeof(double));
	AL(c->mean, sizeof(double));
	AL(c->counter, sizeof(int32_t));
	AL(c->counter_pair, 2 * sizeof(unsigned long long));
	if(c->precision == CPIC_FP64)
	{
		AL(c->phi64, ng * sizeof(double));
		AL(c->rho_lo, ng * sizeof(long long));
		AL(c->Ex64, (ng + 3 * (int64_t) g.nx) * sizeof(double));
		AL(c->Ey64, (ng + 3 * (int64_t) g.nx) * sizeof(double));
		AL(c->spec64, ng / g.nx * nh * sizeof(double2));
		AL(c->twx64, g.nx * sizeof(double2));
		AL(c->twy64, g.ny * sizeof(double2));
		cudaMemset(c->Ex64, 0, (ng + 3 * (int64_t) g.nx) * sizeof(double));
		cudaMemset(c->Ey64, 0, (ng + 3 * (int64_t) g.nx) * sizeof(double));
	}
	else
	{
		AL(c->phi32, ng * sizeof(float));
		AL(c->E32, ng * sizeof(float2));
		AL(c->spec32, ng / g.nx * nh * sizeof(float2));
		AL(c->twx32, g.nx * sizeof(float2));
		AL(c->twy32, g.ny * sizeof(float2));
		cudaMemset(c->E32, 0, ng * sizeof(float2));
		c->emap_ok = encode_field_map(c);
	}
#undef AL
	cudaMemset(c->rho, 0, ng * sizeof(long long));
	if(c->rho_lo) cudaMemset(c->rho_lo, 0, ng * sizeof(long long));
	cudaMemset(c->status, 0, sizeof(uint32_t));
	{
		// Green's function cosines as MFT_init computes them
		// (solver.c:257-278) and FFT twiddles exp(-2 pi i k / n), k < n
		// (a power-of-two transform reads the first half).
		std::vector<double> cx(g.nx), cy(g.ny);
		double ccx = 2.0 * M_PI / g.nx, ccy = 2.0 * M_PI / g.ny;
		for(int i = 0; i < g.nx; i++) cx[i] = cos(ccx * i);
		for(int i = 0; i < g.ny; i++) cy[i] = cos(ccy * i);
		cudaMemcpy(c->cosx, cx.data(), g.nx * sizeof(double), cudaMemcpyHostToDevice);
		cudaMemcpy(c->cosy, cy.data(), g.ny * sizeof(double), cudaMemcpyHostToDevice);
		for(int dim = 0; dim < 2; dim++)
		{
			int n = dim == 0 ? g.nx : g.ny;
			std::vector<double2> tw(n);
			std::vector<float2> tf(n);
			for(int k = 0; k < n; k++)
			{
				double a = -2.0 * M_PI * k / n;
				tw[k] = make_double2(cos(a), sin(a));
				tf[k] = make_float2((float) cos(a), (float) sin(a));
			}
			if(c->precision == CPIC_FP64)
				cudaMemcpy(dim == 0 ? c->twx64 : c->twy64, tw.data(), n * sizeof(double2),
						cudaMemcpyHostToDevice);
			else
				cudaMemcpy(dim == 0 ? c->twx32 : c->twy32, tf.data(), n * sizeof(float2),
						cudaMemcpyHostToDevice);
		}
	}
	// the Green's function once, as MFT_init tabulates it (solver.c:257-280)
	if(c->precision == CPIC_FP64)
	{
		if(cudaMalloc(&c->green64, (size_t) nh * g.ny * sizeof(double)) != cudaSuccess)
		{
			r = CPIC_ENOMEM;
			goto fail;
		}
		k_green<double><<<grid_blocks(nh * g.ny), 256>>>(g.nx, g.ny, c->cosx, c->cosy, c->green64);
	}
	else
	{
		if(cudaMalloc(&c->green32, (size_t) nh * g.ny * sizeof(float)) != cudaSuccess)
		{
			r = CPIC_ENOMEM;
			goto fail;
		}
		k_green<float><<<grid_blocks(nh * g.ny), 256>>>(g.nx, g.ny, c->cosx, c->cosy, c->green32);
	}
	if(cudaDeviceSynchronize() != cudaSuccess) { r = CPIC_ECUDA; goto fail; }
	*out = c;
	return CPIC_OK;
fail:
	cpic_destroy(c);
	return r;
}

CPIC_API void cpic_destroy(cpic_ctx_t *c)
{
	if(!c) return;
	cudaStreamSynchronize(c->stream);
	for(int s = 0; s < c->nspecies; s++)
	{
		SpeciesHost &S = c->sp[s];
		free_store(c, S, false);
		free_store(c, S, true);
		cudaFree(S.tiles.base); cudaFree(S.tiles.cap); cudaFree(S.tiles.cnt);
		cudaFree(S.tiles.abase); cudaFree(S.tiles.acap);
		cudaFree(S.tiles.acnt[0]); cudaFree(S.tiles.acnt[1]); cudaFree(S.tiles.order);
		free_spill(S.spill[0]);
		free_spill(S.spill[1]);
	}
	cudaFree(c->rho); cudaFree(c->rho_lo); cudaFree(c->phi64); cudaFree(c->Ex64); cudaFree(c->Ey64);
	cudaFree(c->phi32); cudaFree(c->E32); cudaFree(c->spec64); cudaFree(c->spec32);
	cudaFree(c->twx64); cudaFree(c->twy64); cudaFree(c->twx32); cudaFree(c->twy32);
	cudaFree(c->cosx); cudaFree(c->cosy); cudaFree(c->green64); cudaFree(c->green32); cudaFree(c->mean);
	cudaFree(c->status); cudaFree(c->scratch); cudaFree(c->counter); cudaFree(c->counter_pair);
	if(c->stream) cudaStreamDestroy(c->stream);
	if(c->probe_h) cudaFreeHost(c->probe_h);
	delete c;
}

// Fixed-point scale: the largest power of two keeping every node sum (at
// most sum_s n_s |q_s/e0|, every particle's weights summing to one) below
// 2^62, so that no partial or total sum can wrap.
static void update_qscale(cpic_ctx *c)
{
	double bound = 0.0;
	for(int s = 0; s < c->nspecies; s++)
		bound += (double) c->sp[s].n * fabs(c->sp[s].q / c->p.e0);
	if(bound <= 0.0) bound = 1.0;
	int k = (int) floor(62.0 - log2(bound)) - 1;
	c->qscale = ldexp(1.0, k);
	c->qinv = ldexp(1.0, -k);
	// Mixed form: the deposit is integer weight units (2^-kWeightBits).
	// When every species' charge is an integer multiple (up to 1024) of the
	// smallest one, u, the fixed-point unit is u 2^-kWeightBits and a weight
	// unit of species s is exactly mult_s of them: every sum is then exact,
	// whichever path (tile accumulator, global fallback, spill list) a
	// particle's contribution takes.  Otherwise the scale above is used and
	// each path rounds its own sums.
	c->wq_exact = false;
	if(c->precision == CPIC_MIXED && c->nspecies > 0)
	{
		double u = INFINITY;
		for(int s = 0; s < c->nspecies; s++)
			if(c->sp[s].n > 0) u = std::min(u, fabs(c->sp[s].q / c->p.e0));
		bool ok = u > 0.0 && std::isfinite(u);
		double units = 0.0;
		for(int s = 0; s < c->nspecies && ok; s++)
		{
			double r = fabs(c->sp[s].q / c->p.e0) / u;
			double mi = nearbyint(r);
			if(mi < 1.0 || mi > 1024.0 || fabs(r - mi) > 1e-9 * r) ok = false;
			double vq = -c->sp[s].q / c->p.e0;
			c->sp[s].wq_mult = vq < 0 ? -mi : mi;
			units += (double) c->sp[s].n * mi;
		}
		if(ok && units * ldexp(1.0, kWeightBits) < ldexp(1.0, 61))
		{
			c->wq_exact = true;
			c->qscale = ldexp(1.0, kWeightBits) / u;
			c->qinv = u * ldexp(1.0, -kWeightBits);
		}
	}
	// FP64 form: remainder word at 2^m finer resolution.  Every remainder
	// is at most 2^(m-1) in magnitude and a node receives at most one per
	// particle, so m = 62 - ceil(log2(N + 1)) keeps its sums below 2^62.
	int64_t ntot = 0;
	for(int s = 0; s < c->nspecies; s++) ntot += c->sp[s].n;
	int m = 62 - (int) ceil(log2((double) ntot + 1.0));
	if(m < 0) m = 0;
	c->qlo_mul = ldexp(1.0, m);
	c->qinv_lo = ldexp(1.0, -k - m);
}

CPIC_API int cpic_add_species(cpic_ctx_t *c, double q, double m, int64_t n,
		const double *x, const double *y, const double *ux, const double *uy)
{
	if(!c || n < 0 || n >= INT32_MAX || !(m != 0.0) || c->nspecies >= kMaxSpecies)
		return CPIC_EINVAL;
	if(n > 0 && (!x || !y || !ux || !uy)) return CPIC_EINVAL;
	if(c->prepared) return CPIC_ESTATE;
	int r;
	cudaStream_t st = c->stream;

	// staging upload in the FP64 spill layout, checked on the device in one
	// pass that also numbers the particles and wraps Y: x in [0, Lx] (the
	// reference's global exchange never wraps X, comm_plasma.c:826-870),
	// finite y, ux, uy; largest |u| component for the halo
	Spill stg;
	memset(&stg, 0, sizeof(stg));
	if((r = alloc_spill(stg, (int32_t) std::max<int64_t>(n, 1), st))) return r;
	double vmax = 0.0;
	if(n > 0)
	{
		CK(cudaMemcpyAsync(stg.x, x, n * sizeof(double), cudaMemcpyHostToDevice, st));
		CK(cudaMemcpyAsync(stg.y, y, n * sizeof(double), cudaMemcpyHostToDevice, st));
		CK(cudaMemcpyAsync(stg.ux, ux, n * sizeof(double), cudaMemcpyHostToDevice, st));
		CK(cudaMemcpyAsync(stg.uy, uy, n * sizeof(double), cudaMemcpyHostToDevice, st));
		unsigned long long *chk = reinterpret_cast<unsigned long long *>(c->counter_pair);
		CK(cudaMemsetAsync(chk, 0, 2 * sizeof(unsigned long long), st));
		k_upload_check<<<grid_blocks(n, 256, 8 * 152), 256, 0, st>>>(n, stg, c->p.Lx, c->p.Ly, chk);
		unsigned long long h[2];
		CK(cudaMemcpyAsync(h, chk, sizeof(h), cudaMemcpyDeviceToHost, st));
		CK(cudaStreamSynchronize(st));
		if(h[0])
		{
			free_spill(stg);
			return CPIC_EINVAL;
		}
		memcpy(&vmax, &h[1], sizeof(double));
	}

	int s = c->nspecies;
	SpeciesHost &S = c->sp[s];
	memset((void *) &S, 0, sizeof(S));
	S.q = q; S.m = m; S.n = n;
	S.vmax = vmax;
	// the fused kernel's instance when the caller left it to the library:
	// 1 particle per thread (chunks of 256) while every species has fewer
	// than kSmallTile particles per tile, else 2 (chunks of 512).  A tile's
	// last main-region chunk and its arrivals chunk are partial, and on
	// small tiles they and the latency between chunks dominate: the FP64
	// two-species 512x512 workload (about 1,100 particles per 8x8 tile and
	// species) steps in 1.498 ms with 1, 1.678 ms with 2; two-stream 2048x2048
	// (102,400 per tile) is fastest with 2.
	if(c->p.particles_per_thread <= 0)
	{
		constexpr int64_t kSmallTile = 4096;
		bool small = n / std::max(1, c->ntiles) < kSmallTile;
		for(int k = 0; k < c->nspecies; k++)
			small = small && c->sp[k].n / std::max(1, c->ntiles) < kSmallTile;
		c->ppt = small ? 1 : kPPT;
	}
	int nt = c->ntiles;
	CK(cudaMalloc(&S.tiles.base, nt * sizeof(int64_t)));
	CK(cudaMalloc(&S.tiles.cap, nt * sizeof(int32_t)));
	CK(cudaMalloc(&S.tiles.cnt, nt * sizeof(int32_t)));
	CK(cudaMalloc(&S.tiles.abase, nt * sizeof(int64_t)));
	CK(cudaMalloc(&S.tiles.acap, nt * sizeof(int32_t)));
	CK(cudaMalloc(&S.tiles.acnt[0], nt * sizeof(int32_t)));
	CK(cudaMalloc(&S.tiles.acnt[1], nt * sizeof(int32_t)));
	CK(cudaMalloc(&S.tiles.order, nt * sizeof(int32_t)));
	k_iota<<<grid_blocks(nt), 256, 0, st>>>(nt, S.tiles.order);
	CK(cudaGetLastError());
	CK(cudaMemsetAsync(S.tiles.cnt, 0, nt * sizeof(int32_t), st));
	CK(cudaMemsetAsync(S.tiles.acnt[0], 0, nt * sizeof(int32_t), st));
	CK(cudaMemsetAsync(S.tiles.acnt[1], 0, nt * sizeof(int32_t), st));
	// room for an eighth of the species to overflow between two host checks
	int32_t scap = (int32_t) std::max<int64_t>(65536, n / 8);
	const int cu = c->precision == CPIC_MIXED ? 1 : 0;
	if((r = alloc_spill(S.spill[0], scap, st, cu))) return r;
	if((r = alloc_spill(S.spill[1], scap, st, cu))) return r;
	c->nspecies++;

	// counting sort of the staged particles into the tiles
	update_qscale(c);
	r = rebuild_species(c, s, true, &stg, n);
	free_spill(stg);
	if(r) return r;
	// halo: a particle displaced by at most D cells in a step deposits
	// into its tile's accumulator when H >= ceil(D).  Take the largest H up
	// to 1.2 D + 1 (room for the plasma to heat) that keeps as many fused
	// kernel blocks resident per SM as H = ceil(D) does.  Faster particles
	// deposit through global memory: correct, slower.
	vmax = 0.0;
	for(int k = 0; k < c->nspecies; k++) vmax = std::max(vmax, c->sp[k].vmax);
	if(c->p.halo <= 0)
	{
		double D = vmax * c->p.dt * std::max(c->g.idx, c->g.idy);
		int hmin = std::max(1, std::min((int) ceil(D), c->g.tx));
		int H = std::max(hmin, std::min((int) ceil(1.2 * D) + 1, c->g.tx));
		if(c->precision == CPIC_MIXED)
		{
			int target = push_mix_blocks_per_sm(push_smem_h(c, hmin), c->p.track_ids != 0, c->ppt, c->g.pow2 != 0);
			while(H > hmin && push_mix_blocks_per_sm(push_smem_h(c, H), c->p.track_ids != 0, c->ppt, c->g.pow2 != 0)
					< target)
				H--;
		}
		c->g.halo = H;
	}
	return s;
}

CPIC_API int cpic_pre_step(cpic_ctx_t *c)
{
	if(!c) return CPIC_EINVAL;
	if(c->prepared) return CPIC_ESTATE;
	int r = plasma_stage_async(c, true);
	if(r) return r;
	if((r = field_stage_async(c))) return r;
	if((r = step_check(c))) return r;
	c->prepared = true;
	c->iter = 0;
	return CPIC_OK;
}

CPIC_API int cpic_stage_field_E(cpic_ctx_t *c)
{
	if(!c) return CPIC_EINVAL;
	int r = field_stage_async(c);
	if(r) return r;
	return check_status(c);
}

CPIC_API int cpic_stage_plasma(cpic_ctx_t *c)
{
	if(!c) return CPIC_EINVAL;
	if(!c->prepared) return CPIC_ESTATE;
	int r = plasma_stage_async(c, false);
	if(r) return r;
	c->iter++;
	return step_check(c);
}

CPIC_API int cpic_step(cpic_ctx_t *c)
{
	if(!c) return CPIC_EINVAL;
	if(!c->prepared) return CPIC_ESTATE;
	if(c->p.cycles > 0 && c->iter >= c->p.cycles) return CPIC_EDONE;
	int r = field_stage_async(c);
	if(r) return r;
	if((r = plasma_stage_async(c, false))) return r;
	c->iter++;
	return step_check(c);
}

static int run_steps(cpic_ctx *c, int64_t nsteps)
{
	for(int64_t k = 0; k < nsteps; k++)
	{
		if(c->p.cycles > 0 && c->iter >= c->p.cycles) return CPIC_EDONE;
		int r = field_stage_async(c);
		if(r) return r;
		if((r = plasma_stage_async(c, false))) return r;
		c->iter++;
		if((k & 7) == 7 || k + 1 == nsteps)
			if((r = step_check(c))) return r;
	}
	return CPIC_OK;
}

CPIC_API int cpic_run(cpic_ctx_t *c, int64_t nsteps)
{
	if(!c) return CPIC_EINVAL;
	if(!c->prepared) return CPIC_ESTATE;
	return run_steps(c, nsteps);
}

CPIC_API int64_t cpic_iter(const cpic_ctx_t *c) { return c ? c->iter : -1; }
CPIC_API int cpic_nspecies(const cpic_ctx_t *c) { return c ? c->nspecies : 0; }
CPIC_API int64_t cpic_species_count(const cpic_ctx_t *c, int s)
{
	if(!c || s < 0 || s >= c->nspecies) return -1;
	return c->sp[s].n;
}

CPIC_API int cpic_get_particles(cpic_ctx_t *c, int s, double *x, double *y, double *ux,
		double *uy)
{
	if(!c || s < 0 || s >= c->nspecies) return CPIC_EINVAL;
	int r = normalize(c);
	if(r) return r;
	int64_t n = c->sp[s].n;
	int nt = c->ntiles;
	// scratch: the four FP64 columns, then the per-tile prefix (store order)
	r = ensure_scratch(c, 4 * (size_t) std::max<int64_t>(n, 1) + nt);
	if(r) return r;
	cudaStream_t st = c->stream;
	double *d = c->scratch;
	bool by_id = c->precision == CPIC_FP64 || c->p.track_ids;
	int64_t *prefix = nullptr;
	if(!by_id)
	{
		std::vector<int32_t> cnt(nt);
		std::vector<int64_t> pre(nt);
		CK(cudaMemcpyAsync(cnt.data(), c->sp[s].tiles.cnt, nt * sizeof(int32_t),
				cudaMemcpyDeviceToHost, st));
		CK(cudaStreamSynchronize(st));
		int64_t acc = 0;
		for(int t = 0; t < nt; t++) { pre[t] = acc; acc += cnt[t]; }
		prefix = reinterpret_cast<int64_t *>(d + 4 * std::max<int64_t>(n, 1));
		CK(cudaMemcpyAsync(prefix, pre.data(), nt * sizeof(int64_t), cudaMemcpyHostToDevice, st));
	}
	PushArgs a = make_args(c, c->spill_cur);
	if(c->precision == CPIC_MIXED)
		k_download<Mix><<<c->ntiles, 256, 0, st>>>(a, s, d, d + n, d + 2 * n, d + 3 * n, prefix);
	else
		k_download<F64><<<c->ntiles, 256, 0, st>>>(a, s, d, d + n, d + 2 * n, d + 3 * n, prefix);
	CK(cudaGetLastError());
	double *outs[4] = {x, y, ux, uy};
	for(int k = 0; k < 4; k++)
		if(outs[k] && n > 0)
			CK(cudaMemcpyAsync(outs[k], d + k * n, n * sizeof(double), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	return CPIC_OK;
}

CPIC_API int cpic_set_particles(cpic_ctx_t *c, int s, const double *x, const double *y,
		const double *ux, const double *uy)
{
	if(!c || s < 0 || s >= c->nspecies) return CPIC_EINVAL;
	if(!x || !y || !ux || !uy) return CPIC_EINVAL;
	SpeciesHost &S = c->sp[s];
	int64_t n = S.n;
	for(int64_t i = 0; i < n; i++)
		if(!(x[i] >= 0.0 && x[i] <= c->p.Lx) || !(y[i] >= 0.0 && y[i] <= c->p.Ly))
			return CPIC_EINVAL;
	cudaStream_t st = c->stream;
	Spill stg;
	memset(&stg, 0, sizeof(stg));
	int r = alloc_spill(stg, (int32_t) std::max<int64_t>(n, 1), st);
	if(r) return r;
	if(n > 0)
	{
		CK(cudaMemcpyAsync(stg.x, x, n * sizeof(double), cudaMemcpyHostToDevice, st));
		CK(cudaMemcpyAsync(stg.y, y, n * sizeof(double), cudaMemcpyHostToDevice, st));
		CK(cudaMemcpyAsync(stg.ux, ux, n * sizeof(double), cudaMemcpyHostToDevice, st));
		CK(cudaMemcpyAsync(stg.uy, uy, n * sizeof(double), cudaMemcpyHostToDevice, st));
		k_iota<<<grid_blocks(n), 256, 0, st>>>(n, stg.id);
	}
	r = rebuild_species(c, s, true, &stg, n);
	free_spill(stg);
	return r;
}

CPIC_API int cpic_gather_E(cpic_ctx_t *c, int s, double *ex, double *ey)
{
	if(!c || s < 0 || s >= c->nspecies) return CPIC_EINVAL;
	if(c->precision == CPIC_MIXED && !c->p.track_ids) return CPIC_EINVAL;
	int64_t n = c->sp[s].n;
	int r = normalize(c);
	if(r) return r;
	r = ensure_scratch(c, 2 * (size_t) std::max<int64_t>(n, 1));
	if(r) return r;
	cudaStream_t st = c->stream;
	SpeciesHost &S = c->sp[s];
	if(c->precision == CPIC_MIXED)
		launch_gather_mix_tiles(c->g, S.mix, S.tiles.base, S.tiles.cnt, c->ntiles, c->E32,
				c->scratch, c->scratch + n, st);
	else
		launch_gather_f64_tiles(c->g, S.f64, S.tiles.base, S.tiles.cnt, c->ntiles, c->Ex64,
				c->Ey64, c->scratch, c->scratch + n, st);
	CK(cudaGetLastError());
	if(ex) CK(cudaMemcpyAsync(ex, c->scratch, n * sizeof(double), cudaMemcpyDeviceToHost, st));
	if(ey) CK(cudaMemcpyAsync(ey, c->scratch + n, n * sizeof(double), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	return CPIC_OK;
}

CPIC_API int cpic_get_rho(cpic_ctx_t *c, double *rho)
{
	if(!c || !rho) return CPIC_EINVAL;
	int64_t ng = (int64_t) c->g.nx * c->g.ny;
	int r = ensure_scratch(c, ng);
	if(r) return r;
	k_rho_to_f64<<<grid_blocks(ng), 256, 0, c->stream>>>(ng, c->rho, c->qinv, c->rho_lo,
			c->qinv_lo, c->scratch);
	CK(cudaMemcpyAsync(rho, c->scratch, ng * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return CPIC_OK;
}

CPIC_API int cpic_set_rho(cpic_ctx_t *c, const double *rho)
{
	if(!c || !rho) return CPIC_EINVAL;
	int64_t ng = (int64_t) c->g.nx * c->g.ny;
	int r = ensure_scratch(c, ng);
	if(r) return r;
	CK(cudaMemcpyAsync(c->scratch, rho, ng * sizeof(double), cudaMemcpyHostToDevice, c->stream));
	k_f64_to_rho<<<grid_blocks(ng), 256, 0, c->stream>>>(ng, c->scratch, c->qscale, c->rho,
			c->qlo_mul, c->rho_lo);
	CK(cudaStreamSynchronize(c->stream));
	return CPIC_OK;
}

CPIC_API int cpic_get_phi(cpic_ctx_t *c, double *phi)
{
	if(!c || !phi) return CPIC_EINVAL;
	int64_t ng = (int64_t) c->g.nx * c->g.ny;
	if(c->precision == CPIC_FP64)
	{
		CK(cudaMemcpy(phi, c->phi64, ng * sizeof(double), cudaMemcpyDeviceToHost));
		return CPIC_OK;
	}
	std::vector<float> tmp(ng);
	CK(cudaMemcpy(tmp.data(), c->phi32, ng * sizeof(float), cudaMemcpyDeviceToHost));
	for(int64_t i = 0; i < ng; i++) phi[i] = tmp[i];
	return CPIC_OK;
}

CPIC_API int cpic_get_E(cpic_ctx_t *c, double *ex, double *ey)
{
	if(!c) return CPIC_EINVAL;
	int64_t nx = c->g.nx, ng = nx * c->g.ny, ne = ng + nx;
	CK(cudaStreamSynchronize(c->stream));
	if(c->precision == CPIC_FP64)
	{
		if(ex) CK(cudaMemcpy(ex, c->Ex64, ne * sizeof(double), cudaMemcpyDeviceToHost));
		if(ey) CK(cudaMemcpy(ey, c->Ey64, ne * sizeof(double), cudaMemcpyDeviceToHost));
		return CPIC_OK;
	}
	std::vector<float2> tmp(ng);
	CK(cudaMemcpy(tmp.data(), c->E32, ng * sizeof(float2), cudaMemcpyDeviceToHost));
	for(int64_t i = 0; i < ne; i++)
	{
		float2 v = tmp[i % ng];
		if(ex) ex[i] = v.x;
		if(ey) ey[i] = v.y;
	}
	return CPIC_OK;
}

CPIC_API int cpic_set_E(cpic_ctx_t *c, const double *ex, const double *ey)
{
	if(!c || !ex || !ey) return CPIC_EINVAL;
	int64_t nx = c->g.nx, ng = nx * c->g.ny, ne = ng + nx;
	if(c->precision == CPIC_FP64)
	{
		CK(cudaMemcpy(c->Ex64, ex, ne * sizeof(double), cudaMemcpyHostToDevice));
		CK(cudaMemcpy(c->Ey64, ey, ne * sizeof(double), cudaMemcpyHostToDevice));
		return CPIC_OK;
	}
	std::vector<float2> tmp(ng);
	for(int64_t i = 0; i < ng; i++) tmp[i] = make_float2((float) ex[i], (float) ey[i]);
	CK(cudaMemcpy(c->E32, tmp.data(), ng * sizeof(float2), cudaMemcpyHostToDevice));
	return CPIC_OK;
}

CPIC_API int cpic_cell_counts(cpic_ctx_t *c, int64_t *counts)
{
	if(!c || !counts) return CPIC_EINVAL;
	int64_t ng = (int64_t) c->g.nx * c->g.ny;
	int r = normalize(c);
	if(r) return r;
	r = ensure_scratch(c, ng);
	if(r) return r;
	cudaStream_t st = c->stream;
	unsigned long long *d = (unsigned long long *) c->scratch;
	CK(cudaMemsetAsync(d, 0, ng * sizeof(unsigned long long), st));
	PushArgs a = make_args(c, c->spill_cur);
	for(int s = 0; s < c->nspecies; s++)
	{
		if(c->precision == CPIC_MIXED)
			k_cell_counts<Mix><<<c->ntiles, 256, 0, st>>>(a, s, d);
		else
			k_cell_counts<F64><<<c->ntiles, 256, 0, st>>>(a, s, d);
	}
	CK(cudaGetLastError());
	CK(cudaMemcpyAsync(counts, d, ng * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	return CPIC_OK;
}

CPIC_API int cpic_diag(cpic_ctx_t *c, double *out)
{
	if(!c || !out) return CPIC_EINVAL;
	int nt = c->ntiles, ny = c->g.ny;
	size_t need = std::max<size_t>(2 * (size_t) ny, 3 * (size_t) nt);
	int r = normalize(c);
	if(r) return r;
	r = ensure_scratch(c, need);
	if(r) return r;
	cudaStream_t st = c->stream;
	std::vector<double> h(need);
	k_field_energy<<<ny, 256, 0, st>>>(c->g, c->Ex64, c->Ey64,
			c->precision == CPIC_MIXED ? c->E32 : nullptr, c->rho, c->scratch);
	CK(cudaMemcpyAsync(h.data(), c->scratch, 2 * ny * sizeof(double), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	double we = 0.0, q = 0.0;
	for(int i = 0; i < ny; i++) { we += h[2 * i]; q += h[2 * i + 1]; }
	double ke = 0.0, px = 0.0, py = 0.0;
	PushArgs a = make_args(c, c->spill_cur);
	for(int s = 0; s < c->nspecies; s++)
	{
		if(c->precision == CPIC_MIXED)
			k_kinetic<Mix><<<nt, 256, 0, st>>>(a, s, c->sp[s].m, c->scratch);
		else
			k_kinetic<F64><<<nt, 256, 0, st>>>(a, s, c->sp[s].m, c->scratch);
		CK(cudaMemcpyAsync(h.data(), c->scratch, 3 * nt * sizeof(double), cudaMemcpyDeviceToHost, st));
		CK(cudaStreamSynchronize(st));
		for(int t = 0; t < nt; t++) { ke += h[3 * t]; px += h[3 * t + 1]; py += h[3 * t + 2]; }
	}
	out[0] = 0.5 * c->p.e0 * we * c->g.dx * c->g.dy;
	out[1] = ke;
	out[2] = q * c->qinv * c->g.dx * c->g.dy;
	out[3] = px;
	out[4] = py;
	return CPIC_OK;
}

CPIC_API int cpic_field_energy(cpic_ctx_t *c, double *out)
{
	if(!c || !out) return CPIC_EINVAL;
	int ny = c->g.ny;
	int r = ensure_scratch(c, 2 * (size_t) ny);
	if(r) return r;
	cudaStream_t st = c->stream;
	std::vector<double> h(2 * (size_t) ny);
	k_field_energy<<<ny, 256, 0, st>>>(c->g, c->Ex64, c->Ey64,
			c->precision == CPIC_MIXED ? c->E32 : nullptr, c->rho, c->scratch);
	CK(cudaMemcpyAsync(h.data(), c->scratch, 2 * ny * sizeof(double), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	double we = 0.0, q = 0.0;
	for(int i = 0; i < ny; i++) { we += h[2 * i]; q += h[2 * i + 1]; }
	out[0] = 0.5 * c->p.e0 * we * c->g.dx * c->g.dy;
	out[1] = q * c->qinv * c->g.dx * c->g.dy;
	return CPIC_OK;
}

CPIC_API uint32_t cpic_status_bits(cpic_ctx_t *c)
{
	if(!c) return 0xffffffffu;
	uint32_t st = 0;
	cudaStreamSynchronize(c->stream);
	cudaMemcpy(&st, c->status, sizeof(st), cudaMemcpyDeviceToHost);
	return st;
}

// Re-lays the particle store out with the given capacity slack (a
// counting-sort rebuild from the current tiles and spill list).
CPIC_API int cpic_compact(cpic_ctx_t *c, int32_t slack_pct)
{
	if(!c || slack_pct < 0 || slack_pct > 1000) return CPIC_EINVAL;
	if(!c->prepared) return CPIC_ESTATE;
	int r = normalize(c);
	if(r) return r;
	CK(cudaStreamSynchronize(c->stream));
	c->slack_pct = slack_pct;
	for(int s = 0; s < c->nspecies; s++)
		if((r = rebuild_species(c, s, false, nullptr, 0)))
			return r;
	CK(cudaStreamSynchronize(c->stream));
	return check_status(c);
}

// One warp waits on an mbarrier phase that cannot complete: thread 0 arms it
// for 16 bytes of a bulk copy that is never issued, so no copy is in flight
// and the wait can only expire.  The status word records ST_TIMEOUT.
__global__ void k_wait_selftest(uint32_t polls, uint32_t *status)
{
	__shared__ __align__(8) uint64_t bar;
	if(threadIdx.x == 0)
	{
		mbar_init(&bar, 1);
		fence_mbar_init();
	}
	__syncthreads();
	if(threadIdx.x == 0)
		mbar_arrive_expect_tx(&bar, 16);
	__syncwarp();
	mbar_wait_bounded(&bar, 0, status, polls);
}

CPIC_API int cpic_selftest_wait(uint32_t polls)
{
	if(polls == 0 || polls > kWaitPolls) return CPIC_EINVAL;
	int ndev = 0;
	if(cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return CPIC_ENODEV;
	uint32_t *d = nullptr, st = 0;
	cudaStream_t s = nullptr;
	int r = CPIC_OK;
	if(cudaMalloc((void **) &d, sizeof(uint32_t)) != cudaSuccess) return CPIC_ENOMEM;
	if(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess
			|| cudaMemsetAsync(d, 0, sizeof(uint32_t), s) != cudaSuccess)
		r = CPIC_ECUDA;
	if(r == CPIC_OK)
	{
		k_wait_selftest<<<1, 32, 0, s>>>(polls, d);
		if(cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess
				|| cudaMemcpy(&st, d, sizeof(st), cudaMemcpyDeviceToHost) != cudaSuccess)
			r = CPIC_ECUDA;
	}
	if(s) cudaStreamDestroy(s);
	cudaFree(d);
	if(r != CPIC_OK) return r;
	return (st & ST_TIMEOUT) ? CPIC_ETIMEOUT : CPIC_OK;
}

CPIC_API int cpic_time_steps(cpic_ctx_t *c, int64_t nsteps, double *ms_total, double *ms_plasma,
		double *ms_field)
{
	if(!c || nsteps <= 0) return CPIC_EINVAL;
	if(!c->prepared) return CPIC_ESTATE;
	cudaStream_t st = c->stream;
	std::vector<cudaEvent_t> ev(2 * nsteps + 2 + 2 * nsteps);
	for(auto &e : ev) CK(cudaEventCreate(&e));
	int r = CPIC_OK;
	CK(cudaStreamSynchronize(st));
	CK(cudaEventRecord(ev[0], st));
	for(int64_t k = 0; k < nsteps; k++)
	{
		cudaEvent_t f0 = ev[2 + 2 * nsteps + 2 * k];
		cudaEvent_t f1 = ev[2 + 2 * nsteps + 2 * k + 1];
		CK(cudaEventRecord(f0, st));
		if((r = field_stage_async(c))) break;
		CK(cudaEventRecord(f1, st));
		if((r = plasma_stage_async(c, false, ev[2 + 2 * k], ev[2 + 2 * k + 1]))) break;
		c->iter++;
	}
	CK(cudaEventRecord(ev[1], st));
	CK(cudaEventSynchronize(ev[1]));
	float tot = 0.0f;
	double sp = 0.0, sf = 0.0;
	CK(cudaEventElapsedTime(&tot, ev[0], ev[1]));
	for(int64_t k = 0; k < nsteps; k++)
	{
		float a = 0.0f, b = 0.0f;
		CK(cudaEventElapsedTime(&a, ev[2 + 2 * k], ev[2 + 2 * k + 1]));
		CK(cudaEventElapsedTime(&b, ev[2 + 2 * nsteps + 2 * k], ev[2 + 2 * nsteps + 2 * k + 1]));
		sp += a;
		sf += b;
	}
	for(auto &e : ev) cudaEventDestroy(e);
	if(ms_total) *ms_total = tot;
	if(ms_plasma) *ms_plasma = sp;
	if(ms_field) *ms_field = sf;
	if(r) return r;
	return step_check(c);
}

CPIC_API int cpic_layout_stats(const cpic_ctx_t *c, int64_t *out)
{
	if(!c || !out) return CPIC_EINVAL;
	out[0] = c->last_spill;
	out[1] = c->rebuilds;
	out[2] = c->slack_pct;
	out[3] = 0;
	if(c->nspecies > 0)
	{
		if(c->precision == CPIC_MIXED)
			out[3] = push_mix_blocks_per_sm(push_smem(c), c->p.track_ids != 0, c->ppt, c->g.pow2 != 0);
		else
			out[3] = push_f64_blocks_per_sm(push_smem(c), c->ppt);
	}
	return CPIC_OK;
}

CPIC_API int cpic_field_tile_copy(const cpic_ctx_t *c, int32_t *mode)
{
	if(!c || !mode) return CPIC_EINVAL;
	*mode = c->emap_ok ? 1 : 0;
	return CPIC_OK;
}

CPIC_API int cpic_tile_info(const cpic_ctx_t *c, int32_t *out)
{
	if(!c || !out) return CPIC_EINVAL;
	out[0] = c->g.tx;
	out[1] = c->g.ty;
	out[2] = c->g.halo;
	out[3] = c->slack_pct;
	return CPIC_OK;
}

} // extern "C"

// ------------------------------------------------------------------------
// Ensembles: many independent runs stepped by one CUDA graph.
//
// Every step of a run is a fixed sequence of asynchronous launches whose
// arguments depend only on the iteration being 0 or not and on the parity
// of the double-buffered spill list, so two steps of every run (iteration
// >= 1) are captured once -- each run on its own stream, forked from and
// joined into one origin stream, i.e. independent branches of one graph --
// and the executable graph is relaunched.  The host checks the runs'
// status words every 4 steps; a run whose tile layout had to be rebuilt
// (new store pointers) triggers one re-capture.

// Per run: its status word and the spill list each species wrote last.
struct EnsProbe {
	const uint32_t *status;
	const int32_t *spill[kMaxSpecies];
	int nspecies;
};

// out[2 i] = status bits of run i, out[2 i + 1] = its largest spill count.
__global__ void k_ens_status(int nruns, const EnsProbe *pr, int32_t *out)
{
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < nruns; i += gridDim.x * blockDim.x)
	{
		int32_t m = 0;
		for(int s = 0; s < pr[i].nspecies; s++) m = max(m, *pr[i].spill[s]);
		out[2 * i] = (int32_t) *pr[i].status;
		out[2 * i + 1] = m;
	}
}

struct cpic_ensemble {
	std::vector<cpic_ctx *> runs;
	EnsProbe *probe_d = nullptr;
	int32_t *probe_out_d = nullptr;
	std::vector<EnsProbe> probe_h;
	std::vector<int32_t> probe_out_h;
	cudaStream_t origin = nullptr;
	cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
	std::vector<cudaEvent_t> join;
	cudaGraphExec_t exec = nullptr;
	bool stale = false;       // a run's layout changed since the capture
	int captures = 0;
	// what the graph's launches hold by value: every run's current store,
	// tile layout and spill-list parity at the capture
	std::vector<const void *> sig;
};

static std::vector<const void *> ens_sig(const cpic_ensemble *e)
{
	std::vector<const void *> v;
	for(const cpic_ctx *c : e->runs)
	{
		v.push_back(reinterpret_cast<const void *>((uintptr_t) c->spill_cur));
		for(int s = 0; s < c->nspecies; s++)
		{
			v.push_back(c->sp[s].f64.x);
			v.push_back(c->sp[s].mix.cell);
			v.push_back(c->sp[s].tiles.base);
		}
	}
	return v;
}

static void ens_drop_graph(cpic_ensemble *e)
{
	if(e->exec) cudaGraphExecDestroy(e->exec);
	e->exec = nullptr;
}

static int ens_capture(cpic_ensemble *e)
{
	cudaGraph_t graph = nullptr;
	// two steps swap every spill list twice: the signature after the
	// capture is the one before it
	e->sig = ens_sig(e);
	CK(cudaStreamBeginCapture(e->origin, cudaStreamCaptureModeRelaxed));
	int r = CPIC_OK;
	if(cudaEventRecord(e->fork, e->origin) != cudaSuccess) r = CPIC_ECUDA;
	for(size_t i = 0; i < e->runs.size() && r == CPIC_OK; i++)
	{
		cpic_ctx *c = e->runs[i];
		if(cudaStreamWaitEvent(c->stream, e->fork, 0) != cudaSuccess) { r = CPIC_ECUDA; break; }
		for(int k = 0; k < 2 && r == CPIC_OK; k++)
		{
			r = field_stage_async(c);
			if(r == CPIC_OK) r = plasma_stage_async(c, false);
		}
		if(r == CPIC_OK && (cudaEventRecord(e->join[i], c->stream) != cudaSuccess
				|| cudaStreamWaitEvent(e->origin, e->join[i], 0) != cudaSuccess))
			r = CPIC_ECUDA;
	}
	cudaError_t ce = cudaStreamEndCapture(e->origin, &graph);
	if(r) { if(graph) cudaGraphDestroy(graph); return r; }
	if(ce != cudaSuccess) return CPIC_ECUDA;
	e->captures++;
	e->stale = false;
	if(e->exec)
	{
		// same launches with new pointers (a rebuilt layout): update the
		// executable graph in place when the topology allows it
		cudaGraphExecUpdateResultInfo info;
		if(cudaGraphExecUpdate(e->exec, graph, &info) == cudaSuccess)
		{
			cudaGraphDestroy(graph);
			return CPIC_OK;
		}
		cudaGetLastError();
		ens_drop_graph(e);
	}
	ce = cudaGraphInstantiate(&e->exec, graph, 0);
	cudaGraphDestroy(graph);
	if(ce != cudaSuccess) { e->exec = nullptr; return CPIC_ECUDA; }
	return CPIC_OK;
}

static int status_code(uint32_t st)
{
	if(st & ST_SPILL_FULL) return CPIC_ECAPACITY;
	if(st & ST_UMAX) return CPIC_EUMAX;
	if(st & ST_NAN) return CPIC_ENAN;
	if(st & ST_RANGE) return CPIC_EINVAL;
	if(st & ST_TIMEOUT) return CPIC_ETIMEOUT;
	return CPIC_OK;
}

// Status of every run, gathered on the device into one small read-back
// after the origin stream's work; rebuilds the tile layout of runs that
// spilled (the graph must then be captured again).
static int ens_check(cpic_ensemble *e, bool *rebuilt)
{
	int nr = (int) e->runs.size();
	*rebuilt = false;
	for(int i = 0; i < nr; i++)
	{
		cpic_ctx *c = e->runs[i];
		EnsProbe &p = e->probe_h[i];
		p.status = c->status;
		p.nspecies = c->nspecies;
		for(int s = 0; s < c->nspecies; s++) p.spill[s] = c->sp[s].spill[c->spill_cur].count;
	}
	CK(cudaMemcpyAsync(e->probe_d, e->probe_h.data(), nr * sizeof(EnsProbe),
			cudaMemcpyHostToDevice, e->origin));
	k_ens_status<<<(nr + 255) / 256, 256, 0, e->origin>>>(nr, e->probe_d, e->probe_out_d);
	CK(cudaMemcpyAsync(e->probe_out_h.data(), e->probe_out_d, 2 * nr * sizeof(int32_t),
			cudaMemcpyDeviceToHost, e->origin));
	CK(cudaStreamSynchronize(e->origin));
	for(int i = 0; i < nr; i++)
	{
		int r = status_code((uint32_t) e->probe_out_h[2 * i]);
		if(r) return r;
	}
	for(int i = 0; i < nr; i++)
	{
		if(e->probe_out_h[2 * i + 1] <= 0) continue;
		cpic_ctx *c = e->runs[i];
		bool rb = false;
		int r = rebuild_if_spilled(c, false, &rb);
		if(r) return r;
		*rebuilt = *rebuilt || rb;
	}
	return CPIC_OK;
}

extern "C" {

CPIC_API int cpic_ensemble_create(cpic_ctx_t *const *runs, int32_t nruns, cpic_ensemble_t **out)
{
	if(!runs || nruns <= 0 || !out) return CPIC_EINVAL;
	*out = nullptr;
	for(int32_t i = 0; i < nruns; i++)
		if(!runs[i] || !runs[i]->prepared) return CPIC_ESTATE;
	cpic_ensemble *e = new cpic_ensemble();
	e->runs.assign(runs, runs + nruns);
	e->join.resize(nruns, nullptr);
	int r = CPIC_OK;
	if(cudaStreamCreateWithFlags(&e->origin, cudaStreamNonBlocking) != cudaSuccess
			|| cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming) != cudaSuccess
			|| cudaEventCreate(&e->t0) != cudaSuccess || cudaEventCreate(&e->t1) != cudaSuccess)
		r = CPIC_ECUDA;
	for(int32_t i = 0; i < nruns && r == CPIC_OK; i++)
		if(cudaEventCreateWithFlags(&e->join[i], cudaEventDisableTiming) != cudaSuccess)
			r = CPIC_ECUDA;
	e->probe_h.resize(nruns);
	e->probe_out_h.resize(2 * (size_t) nruns);
	if(r == CPIC_OK && (cudaMalloc(&e->probe_d, nruns * sizeof(EnsProbe)) != cudaSuccess
			|| cudaMalloc(&e->probe_out_d, 2 * nruns * sizeof(int32_t)) != cudaSuccess))
		r = CPIC_ENOMEM;
	if(r) { cpic_ensemble_destroy(e); return r; }
	*out = e;
	return CPIC_OK;
}

CPIC_API void cpic_ensemble_destroy(cpic_ensemble_t *e)
{
	if(!e) return;
	ens_drop_graph(e);
	for(cudaEvent_t ev : e->join) if(ev) cudaEventDestroy(ev);
	if(e->fork) cudaEventDestroy(e->fork);
	if(e->t0) cudaEventDestroy(e->t0);
	if(e->t1) cudaEventDestroy(e->t1);
	if(e->origin) cudaStreamDestroy(e->origin);
	if(e->probe_d) cudaFree(e->probe_d);
	if(e->probe_out_d) cudaFree(e->probe_out_d);
	delete e;
}

CPIC_API int cpic_ensemble_run(cpic_ensemble_t *e, int64_t nsteps, double *ms_graph,
		int32_t *captures)
{
	if(!e || nsteps < 0) return CPIC_EINVAL;
	int r;
	for(cpic_ctx *c : e->runs)
		if(c->p.cycles > 0 && c->iter + nsteps > c->p.cycles) return CPIC_EDONE;
	int64_t done = 0;
	// iteration 0 (the half kick has its own arguments): eagerly, all runs
	// in flight on their own streams
	bool first = false;
	for(cpic_ctx *c : e->runs)
		if(c->iter == 0) first = true;
	if(first && nsteps > 0)
	{
		for(cpic_ctx *c : e->runs)
		{
			if(c->iter != 0) return CPIC_ESTATE;
			if((r = field_stage_async(c)) || (r = plasma_stage_async(c, false))) return r;
			c->iter++;
		}
		bool rebuilt;
		for(cpic_ctx *c : e->runs) CK(cudaStreamSynchronize(c->stream));
		if((r = ens_check(e, &rebuilt))) return r;
		if(rebuilt) e->stale = true;
		done = 1;
	}
	// the graph carries two steps; the spill parity of every run must be
	// the one it was captured with
	float tms = 0.0f;
	int64_t pairs = (nsteps - done) / 2;
	if(pairs > 0)
	{
		// capture again when a run changed since: a rebuilt layout, or an
		// odd number of steps taken outside the graph
		if((!e->exec || e->stale || ens_sig(e) != e->sig) && (r = ens_capture(e))) return r;
		CK(cudaEventRecord(e->t0, e->origin));
		float acc = 0.0f;
		for(int64_t k = 0; k < pairs; k++)
		{
			CK(cudaGraphLaunch(e->exec, e->origin));
			for(cpic_ctx *c : e->runs) c->iter += 2;
			if((k & 1) == 1 || k + 1 == pairs)
			{
				CK(cudaEventRecord(e->t1, e->origin));
				bool rebuilt;
				if((r = ens_check(e, &rebuilt))) return r;
				float part = 0.0f;
				CK(cudaEventElapsedTime(&part, e->t0, e->t1));
				acc += part;
				if(rebuilt)
				{
					if(k + 1 < pairs) { if((r = ens_capture(e))) return r; }
					else e->stale = true;
				}
				CK(cudaEventRecord(e->t0, e->origin));
			}
		}
		tms = acc;
		done += 2 * pairs;
	}
	// an odd last step, eagerly
	if(done < nsteps)
	{
		CK(cudaStreamSynchronize(e->origin));
		for(cpic_ctx *c : e->runs)
		{
			if((r = field_stage_async(c)) || (r = plasma_stage_async(c, false))) return r;
			c->iter++;
		}
		for(cpic_ctx *c : e->runs) CK(cudaStreamSynchronize(c->stream));
		bool rebuilt;
		if((r = ens_check(e, &rebuilt))) return r;
		if(rebuilt) e->stale = true;
	}
	if(ms_graph) *ms_graph = tms;
	if(captures) *captures = e->captures;
	return CPIC_OK;
}

// Tile size (= the re-bin's counting-sort bin width) for a grid and a
// particle count: each candidate runs a seeded two-stream plasma of n
// particles for 3 + 6 steps, the fastest by CUDA events wins.  Results are
// kept per (grid, log2 particles per cell, precision) for the process.
// Times a seeded two-stream plasma (beam speed v0, spread vth, amplitude
// 0.01) with every tile size, and with every particles-per-thread instance
// when tune_ppt (else the context's own choice, p->particles_per_thread);
// the fastest layout wins.  Cached per (grid, log2 particles per cell,
// precision, what was tuned) for the process.
static int autotune(const cpic_params_t *p, int64_t n, double v0, double vth, bool tune_ppt,
		int32_t *tile, int32_t *ppt, double *ms_per_step)
{
	struct Key { int64_t nx, ny; int lppc, prec, tp, fixed_ppt; double ms; int32_t T, P; };
	static std::vector<Key> cache;
	static std::mutex mu;
	double ppc = (double) n / ((double) p->nx * (double) p->ny);
	int lppc = (int) lround(log2(ppc > 0 ? ppc : 1.0));
	int fixed = tune_ppt ? 0 : p->particles_per_thread;
	{
		std::lock_guard<std::mutex> lk(mu);
		for(const Key &k : cache)
			if(k.nx == p->nx && k.ny == p->ny && k.lppc == lppc && k.prec == p->precision
					&& k.tp == (int) tune_ppt && k.fixed_ppt == fixed)
			{
				*tile = k.T;
				if(ppt) *ppt = k.P;
				if(ms_per_step) *ms_per_step = k.ms;
				return CPIC_OK;
			}
	}
	std::vector<double> x(n), y(n), ux(n), uy(n);
	cpic_init_two_stream(1, 0, n, p->Lx, p->Ly, v0, vth, 0.01, x.data(), y.data(), ux.data(),
			uy.data());
	double q = -p->Lx * p->Ly / (double) n;
	int32_t best = 0, best_p = 0;
	double best_ms = INFINITY;
	// tiles of 1 and 2 cells only for grids no larger tile divides
	bool big = false;
	for(int32_t T = 4; T <= 64; T *= 2)
		big = big || (p->nx % T == 0 && p->ny % T == 0 && (p->nx / T) * (p->ny / T) >= 4);
	for(int32_t T = big ? 4 : 1; T <= 64; T *= 2)
	{
		if(p->nx % T || p->ny % T || (p->nx / T) * (p->ny / T) < 4) continue;
		for(int P : kPPTChoices)
		{
			if(!tune_ppt && P != (fixed > 0 ? fixed : kPPT)) continue;
			cpic_params_t q2 = *p;
			q2.tile_x = q2.tile_y = T;
			q2.particles_per_thread = P;
			q2.cycles = 0;
			cpic_ctx_t *c = nullptr;
			int r = cpic_create(&q2, &c);
			if(r) continue;
			double ms = INFINITY;
			if(cpic_add_species(c, q, -q, n, x.data(), y.data(), ux.data(), uy.data()) >= 0
					&& cpic_pre_step(c) == CPIC_OK && cpic_step(c) == CPIC_OK
					&& cpic_time_steps(c, 3, nullptr, nullptr, nullptr) == CPIC_OK)
			{
				double tot = 0.0;
				if(cpic_time_steps(c, 6, &tot, nullptr, nullptr) == CPIC_OK) ms = tot / 6.0;
			}
			cpic_destroy(c);
			if(ms < best_ms) { best_ms = ms; best = T; best_p = P; }
		}
	}
	if(!best) return CPIC_EINVAL;
	{
		std::lock_guard<std::mutex> lk(mu);
		cache.push_back(Key{p->nx, p->ny, lppc, p->precision, (int) tune_ppt, fixed, best_ms, best,
				best_p});
	}
	*tile = best;
	if(ppt) *ppt = best_p;
	if(ms_per_step) *ms_per_step = best_ms;
	return CPIC_OK;
}

CPIC_API int cpic_autotune_tile(const cpic_params_t *p, int64_t n, double v0, double vth,
		int32_t *tile, double *ms_per_step)
{
	if(!p || n <= 0 || !tile) return CPIC_EINVAL;
	return autotune(p, n, v0, vth, false, tile, nullptr, ms_per_step);
}

CPIC_API int cpic_autotune_layout(const cpic_params_t *p, int64_t n, double v0, double vth,
		int32_t *tile, int32_t *particles_per_thread, double *ms_per_step)
{
	if(!p || n <= 0 || !tile || !particles_per_thread) return CPIC_EINVAL;
	return autotune(p, n, v0, vth, true, tile, particles_per_thread, ms_per_step);
}

} // extern "C"
