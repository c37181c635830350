// cpic_common.cuh -- data layout and launch descriptors shared by the
// FP64 and mixed-precision kernel translation units and the host context.
//
// Particle store: per species, structure of arrays partitioned into tiles of
// TX x TY cells.  Tile t owns slots [base[t], base[t] + cap[t]) of every
// array; the first cnt[t] slots hold the particles whose cell lies in the
// tile.  One step moves particles that leave their tile by appending them
// to the destination tile (slot reserved with an atomic on app[D]) and
// compacting the stayers in place; a fix-up pass closes the gap.  Particles
// that find no room go to a spill list that a generic kernel keeps pushing
// until the host rebuilds the layout with a full counting sort.
//
// Charge deposit: 64-bit two's-complement fixed point.  Every contribution
// w*(-q/e0) is rounded to an integer multiple of 1/qscale and summed with
// integer adds, in shared memory per tile and in global memory across
// tiles.  Integer sums are exact and order independent, so the deposit is
// deterministic without float atomics.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cpic {

constexpr int kMaxSpecies = 8;
constexpr int kPushThreads = 256;
constexpr int kPPT = 4;                       // particles per thread per chunk
constexpr int kChunk = kPushThreads * kPPT;   // particles per chunk

// Device status bits (sticky until the host clears them).
enum : uint32_t {
	ST_UMAX = 1u << 0,       // |u| > umax (reference aborts, mover.c:97-137)
	ST_NAN = 1u << 1,        // non-finite particle state
	ST_SPILL_FULL = 1u << 2, // spill list full: particles would be lost
	ST_RANGE = 1u << 3,      // a cell index outside the grid (defensive)
};

struct StoreF64 {
	double *x, *y, *ux, *uy;
	int32_t *id;
};

struct StoreMix {
	int32_t *cell;   // iy * nx + ix
	float *ox, *oy;  // offset inside the cell, [0, 1)
	float *ux, *uy;  // physical velocity
	int32_t *id;     // optional (nullptr when ids are not tracked)
};

struct Tiles {
	int64_t *base;   // first slot of the tile
	int32_t *cap;    // slots owned by the tile
	int32_t *cnt;    // particles at the start of the step
	int32_t *app;    // append cursor (starts at cnt)
	int32_t *stay;   // stayers after the push
};

// Spill list: records that could not be placed in their tile.  Stored in
// the FP64 layout for both precisions (mixed records are widened), plus
// the id.
struct Spill {
	double *x, *y, *ux, *uy;
	int32_t *id;
	int32_t *count;     // number of records
	int32_t capacity;
};

struct Grid {
	int nx, ny;          // cells (= nodes, periodic)
	int tx, ty;          // tile size in cells
	int ntx, nty;        // tiles per dimension
	int halo;            // deposit halo in cells
	double dx, dy, idx, idy, Lx, Ly;
};

// Per-species constants for one step.
struct SpeciesStep {
	double dtqm2;        // 0.5 * dt * q / m (mover.c:211)
	double tz, sz;       // Boris t and s for B along z (mover.c:45-51)
	double umax_x, umax_y;
	double qfix;         // fixed-point units per unit of w: -q/e0 * qscale
	float qfix_f;        // same, FP32 (mixed form)
	float dtqm2_f, tz_f, sz_f;
};

struct PushArgs {
	Grid g;
	int nspecies;
	int iter;            // 0 -> backward half step, no move
	double dt;
	float cdx_f, cdy_f;  // dt/dx, dt/dy (mixed form)
	SpeciesStep sp[kMaxSpecies];
	Tiles tiles[kMaxSpecies];
	StoreF64 f64[kMaxSpecies];
	StoreMix mix[kMaxSpecies];
	Spill spill_out[kMaxSpecies];
	long long *rho;      // ny x nx fixed-point accumulator
	const double *Ex64, *Ey64;     // (ny + 3) x nx, FP64 form
	const float2 *E32;             // ny x nx (Ex, Ey) interleaved, mixed form
	uint32_t *status;
};

struct SpillArgs {
	PushArgs p;
	Spill spill_in[kMaxSpecies];
};

// ---------------------------------------------------------------- helpers

__device__ __forceinline__ int wrapi(int i, int n)
{
	i %= n;
	return i < 0 ? i + n : i;
}

__device__ __forceinline__ void set_status(uint32_t *st, uint32_t bit)
{
	atomicOr(st, bit);
}

// Tile index of a cell.
__device__ __forceinline__ int tile_of(const Grid &g, int cx, int cy)
{
	return (cy / g.ty) * g.ntx + (cx / g.tx);
}

// Shared-memory fixed-point deposit of one particle's four node weights,
// with the node frame relative to the tile origin (tile-local cell rx, ry,
// may lie in the halo).  Falls back to global atomics outside the halo.
template <int NONE>
struct Deposit {};

__device__ __forceinline__ void
dep_global(long long *rho, const Grid &g, int cx, int cy,
		long long w00, long long w01, long long w10, long long w11)
{
	int x0 = wrapi(cx, g.nx), y0 = wrapi(cy, g.ny);
	int x1 = x0 + 1 == g.nx ? 0 : x0 + 1;
	int y1 = y0 + 1 == g.ny ? 0 : y0 + 1;
	atomicAdd((unsigned long long *) &rho[(int64_t) y0 * g.nx + x0], (unsigned long long) w00);
	atomicAdd((unsigned long long *) &rho[(int64_t) y1 * g.nx + x0], (unsigned long long) w01);
	atomicAdd((unsigned long long *) &rho[(int64_t) y0 * g.nx + x1], (unsigned long long) w10);
	atomicAdd((unsigned long long *) &rho[(int64_t) y1 * g.nx + x1], (unsigned long long) w11);
}

// acc is a W x W shared array covering nodes [t0 - H, t0 + T + H] of the
// tile; (rx, ry) is the cell relative to the tile origin.
__device__ __forceinline__ void
dep_tile(long long *acc, int W, int H, const Grid &g, int tx0, int ty0,
		int rx, int ry, long long w00, long long w01, long long w10, long long w11,
		long long *rho)
{
	int lx = rx + H, ly = ry + H;
	if(lx >= 0 && ly >= 0 && lx + 1 < W && ly + 1 < W)
	{
		long long *a = acc + ly * W + lx;
		atomicAdd((unsigned long long *) &a[0], (unsigned long long) w00);
		atomicAdd((unsigned long long *) &a[W], (unsigned long long) w01);
		atomicAdd((unsigned long long *) &a[1], (unsigned long long) w10);
		atomicAdd((unsigned long long *) &a[W + 1], (unsigned long long) w11);
	}
	else
	{
		dep_global(rho, g, tx0 + rx, ty0 + ry, w00, w01, w10, w11);
	}
}

// Add a tile's shared accumulator into the global fixed-point rho.
__device__ __forceinline__ void
flush_tile(const long long *acc, int W, int H, const Grid &g, int tx0, int ty0,
		long long *rho)
{
	for(int i = threadIdx.x; i < W * W; i += blockDim.x)
	{
		long long v = acc[i];
		if(v == 0) continue;
		int gx = wrapi(tx0 - H + i % W, g.nx);
		int gy = wrapi(ty0 - H + i / W, g.ny);
		atomicAdd((unsigned long long *) &rho[(int64_t) gy * g.nx + gx], (unsigned long long) v);
	}
}

// Reserve a slot in the destination tile for a mover: lanes with the same
// destination share one atomic.  Returns the slot or -1 when the tile is
// full (the caller spills).
__device__ __forceinline__ int64_t
reserve_slot(const Tiles &T, int dest, unsigned active)
{
	unsigned peers = __match_any_sync(active, dest);
	int leader = __ffs(peers) - 1;
	int lane = threadIdx.x & 31;
	int rank = __popc(peers & ((1u << lane) - 1));
	int first = 0;
	if(lane == leader)
		first = atomicAdd(&T.app[dest], __popc(peers));
	first = __shfl_sync(peers, first, leader);
	int slot = first + rank;
	if(slot >= T.cap[dest])
		return -1;
	return T.base[dest] + slot;
}

// Append a record to a spill list; false when the list is full.
__device__ __forceinline__ bool
spill_push(const Spill &S, double x, double y, double ux, double uy, int32_t id,
		uint32_t *status)
{
	int k = atomicAdd(S.count, 1);
	if(k >= S.capacity)
	{
		set_status(status, ST_SPILL_FULL);
		return false;
	}
	S.x[k] = x; S.y[k] = y; S.ux[k] = ux; S.uy[k] = uy;
	S.id[k] = id;
	return true;
}

// Block-wide exclusive scan of one flag per thread (kPushThreads threads).
// Returns this thread's offset; *total receives the block sum.  Uses
// `warp_tot` (kPushThreads/32 ints of shared memory); contains two
// __syncthreads.
__device__ __forceinline__ int
block_scan_flag(bool flag, int *warp_tot, int *total)
{
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	unsigned b = __ballot_sync(0xffffffffu, flag);
	int in_warp = __popc(b & ((1u << lane) - 1));
	if(lane == 0) warp_tot[warp] = __popc(b);
	__syncthreads();
	int off = 0, tot = 0;
	#pragma unroll
	for(int w = 0; w < kPushThreads / 32; w++)
	{
		int c = warp_tot[w];
		off += w < warp ? c : 0;
		tot += c;
	}
	__syncthreads();
	*total = tot;
	return off + in_warp;
}

} // namespace cpic

// Launchers implemented in the per-precision translation units.
namespace cpic {
void launch_push_f64(const PushArgs &a, int ntiles, size_t smem, cudaStream_t s);
void launch_spill_f64(const SpillArgs &a, cudaStream_t s);
void launch_gather_f64(const Grid &g, const StoreF64 &st, int64_t n, const double *Ex,
		const double *Ey, double *ex_out, double *ey_out, cudaStream_t s);
void launch_E_f64(const Grid &g, const double *phi, double *Ex, double *Ey, cudaStream_t s);
void launch_poisson_f64(const Grid &g, const long long *rho, double qinv, double *rho_out,
		double2 *spec, const double2 *twx, const double2 *twy, const double *cosx,
		const double *cosy, double *phi, cudaStream_t s);

void launch_push_mix(const PushArgs &a, int ntiles, size_t smem, cudaStream_t s);
void launch_spill_mix(const SpillArgs &a, cudaStream_t s);
void launch_gather_mix(const Grid &g, const StoreMix &st, int64_t n, const float2 *E,
		double *ex_out, double *ey_out, cudaStream_t s);
void launch_E_mix(const Grid &g, const float *phi, float2 *E, cudaStream_t s);
void launch_poisson_mix(const Grid &g, const long long *rho, double qinv, const double *mean,
		float2 *spec, const float2 *twx, const float2 *twy, const double *cosx,
		const double *cosy, float *phi, cudaStream_t s);
} // namespace cpic
