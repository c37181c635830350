// cpic_common.cuh -- data layout and launch descriptors shared by the
// FP64 and mixed-precision kernel translation units and the host context.
//
// Particle store: per species, structure of arrays partitioned into tiles of
// TX x TY cells.  Tile t owns a main region, slots [base[t], base[t] +
// cap[t]) of every array, whose first cnt[t] slots hold particles whose cell
// lies in the tile, and an arrivals region in each of two buffers after the
// main regions.  One step reads a tile's main region and the arrivals the
// previous step left in one buffer, compacts the stayers in place at the
// front of the main region, and appends the particles that leave to their
// destination tile's arrivals in the other buffer (slot reserved with an
// atomic on its count): no pass between steps has to close gaps.  Particles
// that find no room go to a spill list that a generic kernel keeps pushing
// until the host rebuilds the layout with a full counting sort.
//
// Charge deposit: 64-bit two's-complement fixed point in global memory.
// Every contribution is an integer; integer sums are exact and order
// independent, so the deposit is deterministic without float atomics.
// FP64 form: each contribution w*(-q/e0) is rounded to a multiple of
// 1/qscale and summed per tile in 64-bit shared memory.  Mixed form: the
// weights w are rounded to multiples of 2^-kWeightBits and summed per tile
// in 32-bit shared memory (added to global rho and restarted before any
// sum can wrap, which a check every kCheckChunks chunks detects); the
// species charge multiplies the tile sums at the flush.
#pragma once
#include <cstdint>
#include <cuda.h>            // CUtensorMap (the type only; no driver library is linked)
#include <cuda_runtime.h>
#include "cpic_bits.h"

namespace cpic {

constexpr int kMaxSpecies = 8;
// Block shape of the fused particle kernel (build-time knobs).
#ifndef CPIC_PUSH_THREADS
#define CPIC_PUSH_THREADS 256
#endif
#ifndef CPIC_PPT
#define CPIC_PPT 2
#endif
constexpr int kPushThreads = CPIC_PUSH_THREADS;
// Particles per thread per chunk: the default, and the compiled instances of
// the fused kernel a context may choose from (the autotuner times them).
constexpr int kPPT = CPIC_PPT;
constexpr int kPPTChoices[] = {1, 2, 4};
constexpr int kWeightBits = 18;
// Particles per chunk with P particles per thread.
__host__ __device__ constexpr int chunk_of(int P) { return kPushThreads * P; }
// 32-bit shared weight sums: a node gains at most 2^kWeightBits per
// particle, so check_chunks(P) chunks add at most 2^30 to any node; a check
// every check_chunks(P) chunks that finds every node below 2^30 keeps every
// sum below 2^31 until the next check
__host__ __device__ constexpr int check_chunks(int P) { return (1 << (30 - kWeightBits)) / chunk_of(P); }
static_assert(check_chunks(4) >= 1, "chunk too large for 32-bit weight sums");
inline bool ppt_supported(int P) { return P == 1 || P == 2 || P == 4; }

// Device status bits (sticky until the host clears them).
enum : uint32_t {
	ST_UMAX = 1u << 0,       // |u| > umax (reference aborts, mover.c:97-137)
	ST_NAN = 1u << 1,        // non-finite particle state
	ST_SPILL_FULL = 1u << 2, // spill list full: particles would be lost
	ST_RANGE = 1u << 3,      // a cell index outside the grid (defensive)
	ST_TIMEOUT = 1u << 4,    // a bounded wait on a bulk copy expired
};

struct StoreF64 {
	double *x, *y, *ux, *uy;
	int32_t *id;
};

// The mixed form keeps each particle's four floats together (one 16-byte
// load or store each), its packed cell in a column of its own.
struct StoreMix {
	int32_t *cell;   // (cy << lcx) + cx
	float4 *ou;      // (ox, oy, ux, uy): offset inside the cell in [0, 1), velocity
	int32_t *id;     // optional (nullptr when ids are not tracked)
};

// Each tile owns a main region of the store, which its own block compacts in
// place, and two arrivals regions (buffers 0 and 1, abuf1 slots apart) into
// which other blocks append the particles that move in.  A step's fused
// kernel reads the main region and the arrivals that the previous step left
// in buffer r, and appends this step's movers to buffer 1 - r, so no pass
// between steps has to close the gaps the movers leave.
struct Tiles {
	int64_t *base;   // first slot of the tile's main region
	int32_t *cap;    // slots of the main region
	int32_t *cnt;    // particles in the main region at the start of the step
	int64_t *abase;  // first slot of the tile's arrivals region in buffer 0
	int32_t *acap;   // slots of each arrivals region
	int32_t *acnt[2];   // particles in the arrivals region of buffer 0 and 1
	int64_t abuf1;   // slot offset of buffer 1 from buffer 0
	int32_t *order;  // tile taken by block b of the fused kernel (a permutation)
};

// Spill list: records that could not be placed in their tile.  Stored in
// the FP64 layout for both precisions (mixed records are widened), plus
// the id.
struct Spill {
	double *x, *y, *ux, *uy;
	int32_t *id;
	int32_t *count;     // number of records
	int32_t capacity;
	// 0: x, y are positions (uploads); 1: x, y are cell index + in-cell
	// offset in cell units, which carries a mixed-form record exactly
	int32_t cell_units;
};

struct Grid {
	int nx, ny;          // cells (= nodes, periodic)
	int tx, ty;          // tile size in cells
	int ntx, nty;        // tiles per dimension
	int halo;            // deposit halo in cells
	int lcx;             // bits of x in a packed cell index (cy << lcx) + cx:
	                     // ceil(log2 nx), so any nx decodes with a shift and
	                     // a mask
	int ltx, lty;        // log2 of tx, ty (tiles are powers of two)
	uint32_t ntx_mul;    // t / ntx = (t * ntx_mul) >> ntx_sh for a tile
	int ntx_sh;          // index t (bits::div_init)
	int pow2;            // nx and ny are powers of two
	double dx, dy, idx, idy, Lx, Ly;
};

// Per-species constants for one step.
struct SpeciesStep {
	double dtqm2;        // 0.5 * dt * q / m (mover.c:211)
	double tz, sz;       // Boris t and s for B along z (mover.c:45-51)
	double umax_x, umax_y;
	double qfix;         // fixed-point units per unit of w: -q/e0 * qscale
	double qlo_mul;      // FP64 form: 2^m, the scale of the remainder word
	int qlo_exp;         // m
	double wq_scale;     // mixed: fixed-point units per integer weight unit
	long long wq_int;    // the same as an integer when it is one, else 0
	float dtqm2_f, tz_f, sz_f;
	float umax_x_f, umax_y_f;
};

struct PushArgs {
	// mixed form: 2D tensor map of E32 (nx x ny elements of 8 bytes, box
	// (tx + 2) x (ty + 1)) for the fused kernel's field tile; valid when
	// emap_ok.  Kept in the kernel's parameter space, where the tensor
	// copy reads it.
	CUtensorMap emap;
	int emap_ok;
	Grid g;
	int nspecies;
	int arr_r;           // arrivals buffer read by this step (movers go to 1 - arr_r)
	int iter;            // 0 -> backward half step, no move
	double dt;
	float cdx_f, cdy_f;  // dt/dx, dt/dy (mixed form)
	SpeciesStep sp[kMaxSpecies];
	Tiles tiles[kMaxSpecies];
	StoreF64 f64[kMaxSpecies];
	StoreMix mix[kMaxSpecies];
	Spill spill_out[kMaxSpecies];
	long long *rho;      // ny x nx fixed-point accumulator
	long long *rho_lo;   // FP64 form: remainder word, 2^m finer (else null)
	const double *Ex64, *Ey64;     // (ny + 3) x nx, FP64 form
	const float2 *E32;             // ny x nx (Ex, Ey) interleaved, mixed form
	uint32_t *status;
};

struct SpillArgs {
	PushArgs p;
	Spill spill_in[kMaxSpecies];
};

// The arguments of species sp moved to index 0 (the fused kernel is
// launched once per species and reads index 0 only).
inline PushArgs species_args(const PushArgs &a, int sp)
{
	PushArgs b = a;
	b.nspecies = 1;
	b.sp[0] = a.sp[sp];
	b.tiles[0] = a.tiles[sp];
	b.f64[0] = a.f64[sp];
	b.mix[0] = a.mix[sp];
	b.spill_out[0] = a.spill_out[sp];
	return b;
}

// ---------------------------------------------------------------- helpers

// Periodic wrap for a power-of-two extent (any sign of i).
__device__ __forceinline__ int wrap2(int i, int n)
{
	return i & (n - 1);
}

// Periodic wrap for any extent, i in [-n, 2n).
__host__ __device__ __forceinline__ int wrapn(int i, int n)
{
	if(i < 0) i += n;
	else if(i >= n) i -= n;
	return i;
}

// Periodic wrap for any extent and any i (a loop: one or two compares for
// i within one period of the grid).
__host__ __device__ __forceinline__ int wrap_any(int i, int n)
{
	while(i < 0) i += n;
	while(i >= n) i -= n;
	return i;
}

// Periodic wrap for any extent and any i, with a division.
__host__ __device__ __forceinline__ int wrap_mod(int i, int n)
{
	i %= n;
	return i < 0 ? i + n : i;
}

// Row (ty) and column (tx) of tile index t, without a divide instruction
// (bits::div_q: exact for t < 2^30; for a power-of-two ntx it is t >> log2
// ntx).
__device__ __forceinline__ void tile_rc(const Grid &g, int t, int &tx, int &ty)
{
	ty = (int) bits::div_q((uint32_t) t, g.ntx_mul, g.ntx_sh);
	tx = t - ty * g.ntx;
}

__device__ __forceinline__ void set_status(uint32_t *st, uint32_t bit)
{
	atomicOr(st, bit);
}

// Tile index of a cell.
__device__ __forceinline__ int tile_of(const Grid &g, int cx, int cy)
{
	return (cy >> g.lty) * g.ntx + (cx >> g.ltx);
}

// Lanes below this one (the special register: one read, where shifting by
// threadIdx.x & 31 costs four instructions; 0.6 % of the fused kernel's time
// on the two-stream 2048x2048 benchmark).
__device__ __forceinline__ unsigned lanemask_lt()
{
	unsigned m;
	asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
	return m;
}

__device__ __forceinline__ void red_global(long long *p, long long v)
{
	atomicAdd((unsigned long long *) p, (unsigned long long) v);
}

// Fixed-point deposit of one particle's four node values straight into the
// global accumulator (cell (cx, cy) may be outside the grid: wrapped).
__device__ __forceinline__ void
dep_global(long long *rho, const Grid &g, int cx, int cy,
		long long w00, long long w01, long long w10, long long w11)
{
	int x0 = wrap_any(cx, g.nx), y0 = wrap_any(cy, g.ny);
	int x1 = wrapn(x0 + 1, g.nx), y1 = wrapn(y0 + 1, g.ny);
	red_global(&rho[(int64_t) y0 * g.nx + x0], w00);
	red_global(&rho[(int64_t) y1 * g.nx + x0], w01);
	red_global(&rho[(int64_t) y0 * g.nx + x1], w10);
	red_global(&rho[(int64_t) y1 * g.nx + x1], w11);
}

// Two-word variant of dep_global (FP64 form: high and remainder words).
__device__ __forceinline__ void
dep_global2(long long *rho, long long *rlo, const Grid &g, int cx, int cy,
		const long long hi[4], const long long lo[4])
{
	int x0 = wrap_any(cx, g.nx), y0 = wrap_any(cy, g.ny);
	int x1 = wrapn(x0 + 1, g.nx), y1 = wrapn(y0 + 1, g.ny);
	int64_t n[4] = {(int64_t) y0 * g.nx + x0, (int64_t) y1 * g.nx + x0,
		(int64_t) y0 * g.nx + x1, (int64_t) y1 * g.nx + x1};
	for(int c = 0; c < 4; c++)
	{
		red_global(&rho[n[c]], hi[c]);
		red_global(&rlo[n[c]], lo[c]);
	}
}

// Global node index of shared accumulator entry i (frame origin t0 - H).
__device__ __forceinline__ int64_t
frame_node(const Grid &g, int W, int H, int tx0, int ty0, int i)
{
	int gx = wrap_any(tx0 - H + i % W, g.nx);
	int gy = wrap_any(ty0 - H + i / W, g.ny);
	return (int64_t) gy * g.nx + gx;
}

// Split-phase variant: `issue` fires one atomic per distinct destination
// (the leader lane keeps the old value), `finish` broadcasts it; the
// atomics' latency overlaps whatever runs in between.  Whole warp.  One
// match groups the lanes by destination (non-movers share the key -1):
// a fixed handful of instructions, where a loop over the distinct
// destinations (a ballot, a shuffle and an atomic per destination) took
// 5.9 % longer over the whole fused kernel on the two-stream 2048x2048
// benchmark (3.618 against 3.404 ms per launch).
struct Resv { int leader, rank, own; };

__device__ __forceinline__ Resv
warp_reserve_issue(int32_t *cnt, bool move, int dest)
{
	Resv r;
	const unsigned grp = __match_any_sync(0xffffffffu, move ? dest : -1);
	r.leader = __ffs(grp) - 1;
	r.rank = __popc(grp & lanemask_lt());
	r.own = 0;
	if(move && r.rank == 0)
		r.own = atomicAdd(&cnt[dest], __popc(grp));
	return r;
}

__device__ __forceinline__ int
warp_reserve_finish(const Resv &r, bool move)
{
	int first = __shfl_sync(0xffffffffu, r.own, r.leader);
	return move ? first + r.rank : -1;
}

// Warp-aggregated slot reservation for movers: one atomic per distinct
// destination tile in the warp.  Must be called by the whole warp; returns
// the slot within the destination tile for lanes with `move`, else -1.
__device__ __forceinline__ int
warp_reserve(int32_t *cnt, bool move, int dest)
{
	return warp_reserve_finish(warp_reserve_issue(cnt, move, dest), move);
}

// ------------------------------------------------ bulk copies (TMA engine)
//
// One thread streams a chunk of each structure-of-arrays column from global
// into shared memory with cp.async.bulk; completion is counted in bytes on
// an mbarrier that every consumer thread waits on.

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
	return (uint32_t) __cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Order this thread's earlier generic-proxy accesses to shared memory
// before later async-proxy (bulk copy) writes to it.
__device__ __forceinline__ void fence_proxy_async_smem()
{
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
			:: "r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// dst (shared) and src (global) 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
			:: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

// A 2D tile of a tensor map (box dimensions in the map) into shared
// memory; x, y the box's first element and row.  dst 128-byte aligned; x
// times the element size a multiple of 16 bytes.
__device__ __forceinline__ void tensor_g2s_2d(void *dst, const CUtensorMap *map, int x, int y,
		uint64_t *bar)
{
	asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
			" [%0], [%1, {%2, %3}], [%4];"
			:: "r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y),
			"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smem_addr(bar)) : "memory");
}

// One probe of the mbarrier phase of the given parity.  The thread may be
// suspended for a hardware-defined time limit while the phase is pending
// (it wakes as soon as the phase completes).  Measured on the fused kernel
// (2048^2, 20 steps, 3 alternating rounds): 3.643 ms per launch, against
// 3.667 ms with an explicit 100 us suspend-time hint and 3.711 ms with
// test_wait and an exponential nanosleep backoff.
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\t"
			"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
			"selp.u32 %0, 1, 0, p;\n\t}"
			: "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
	return ok != 0;
}

// Probes of a bounded wait before it gives up: each probe suspends the
// thread at most for the hardware's time limit (of the order of a
// microsecond), so a wait that never completes ends within about a second.
constexpr uint32_t kWaitPolls = 1u << 20;

// Wait for the mbarrier phase of the given parity, with an iteration limit:
// on expiry the status word records ST_TIMEOUT and the caller goes on (its
// indices are all clamped, so stale shared data cannot cause an
// out-of-bounds access).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t *status,
		uint32_t polls = kWaitPolls)
{
	for(uint32_t it = 0; it < polls; it++)
		if(mbar_try_wait(bar, parity))
			return true;
	set_status(status, ST_TIMEOUT);
	return false;
}

// Append a record to a spill list; false when the list is full (the count
// then exceeds the capacity, which readers clamp and the host takes as a
// reason to rebuild).
__device__ __forceinline__ bool
spill_push(const Spill &S, double x, double y, double ux, double uy, int32_t id)
{
	int k = atomicAdd(S.count, 1);
	if(k >= S.capacity)
		return false;
	S.x[k] = x; S.y[k] = y; S.ux[k] = ux; S.uy[k] = uy;
	S.id[k] = id;
	return true;
}

} // namespace cpic

#include <initializer_list>
#include <mutex>

namespace cpic {

// One-time set-up per CUDA device.  Kernel attributes such as the dynamic
// shared-memory limit belong to the device that was current when they were
// set, so a context created on another device needs them set again.  run(f)
// calls f() the first time it is made with a given device current and
// remembers success only: a failed f() is retried by the next call.
class PerDeviceOnce {
public:
	template <class F> cudaError_t run(F f)
	{
		int dev = -1;
		cudaError_t e = cudaGetDevice(&dev);
		if(e != cudaSuccess) return e;
		if(dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
		std::lock_guard<std::mutex> lk(m_);
		if((done_ >> dev) & 1ull) return cudaSuccess;
		e = f();
		if(e == cudaSuccess) done_ |= 1ull << dev;
		return e;
	}

private:
	std::mutex m_;
	unsigned long long done_ = 0;
};

// cudaFuncSetAttribute over a list of kernels; the first error, if any.
inline cudaError_t set_max_dyn_smem(std::initializer_list<const void *> fns, int bytes,
		bool carveout = false)
{
	for(const void *f : fns)
	{
		cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
		if(e == cudaSuccess && carveout)
			e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout,
					cudaSharedmemCarveoutMaxShared);
		if(e != cudaSuccess) return e;
	}
	return cudaSuccess;
}

} // namespace cpic

// Launchers implemented in the per-precision translation units.  Those that
// return cudaError_t report a failed one-time kernel set-up; launch errors
// are left for the caller's cudaGetLastError.
namespace cpic {
// ppt: particles per thread of the fused kernel's instance (kPPTChoices)
cudaError_t launch_push_f64(const PushArgs &a, int ntiles, size_t smem, int ppt, cudaStream_t s);
int push_f64_blocks_per_sm(size_t smem, int ppt);
void launch_spill_f64(const SpillArgs &a, cudaStream_t s);
void launch_E_f64(const Grid &g, const double *phi, double *Ex, double *Ey, cudaStream_t s);
cudaError_t launch_poisson_f64(const Grid &g, const long long *rho, double qinv,
		double2 *spec, const double2 *twx, const double2 *twy, const double *cosx,
		const double *cosy, double *phi, cudaStream_t s, const long long *rho_lo, double qinv_lo,
		const double *Gt);

cudaError_t launch_push_mix(const PushArgs &a, int ntiles, size_t smem, int ppt, cudaStream_t s);
// resident blocks per SM of the mixed fused kernel at this dynamic shared
// memory, for a store with or without ids (0 on error)
int push_mix_blocks_per_sm(size_t smem, bool ids, int ppt, bool gp2);
void launch_spill_mix(const SpillArgs &a, cudaStream_t s);
void launch_E_mix(const Grid &g, const float *phi, float2 *E, cudaStream_t s);
cudaError_t launch_poisson_mix(const Grid &g, const long long *rho, double qinv, const long long *rsum,
		float2 *spec, const float2 *twx, const float2 *twy, const double *cosx,
		const double *cosy, float *phi, cudaStream_t s, const float *Gt, double mean0 = 0.0);
} // namespace cpic
