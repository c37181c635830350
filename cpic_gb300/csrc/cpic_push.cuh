// cpic_push.cuh -- the fused particle kernel: field gather, Boris push,
// move, periodic wrap, re-bin and charge deposit, for one tile per block.
//
// Replaces, per step: interpolate_f2p_E (src/interpolate.c:349-404),
// plist_update_r / boris_rotation / move (src/mover.c:22-188), the local
// comm_plasma re-bin and periodic_boundary (src/comm_plasma.c:695-885,
// 1087-1142), interpolate_p2f_rho (src/interpolate.c:282-346) and the rho
// ghost fold (src/comm_field.c:52-136).
//
// Two forms share the kernel skeleton:
//   F64 : positions and velocities in FP64, exact reference arithmetic
//         (this header is compiled with --fmad=false for it); E read from
//         global memory with the reference's index arithmetic, quirks
//         included; 64-bit fixed-point shared accumulator.
//   Mix : int32 cell + FP32 offset, FP32 velocity; E staged per tile in
//         shared memory; 32-bit integer weight accumulator.
//
// Skeleton per block (tile t of species s): the tile's particles -- its main
// region, then the arrivals the previous step left for it -- are read in
// chunks of kChunk; after one barrier per chunk (every load of the chunk has
// landed) each particle is pushed, deposited into the tile's shared
// accumulator, and written back: stayers compacted in place at the front of
// the main region through a shared cursor (a warp reserves its run with one
// shared atomic), movers appended to their destination tile's arrivals in
// the other buffer (one global atomic per distinct destination per warp).
// In-place writes never pass the number of particles read, so they only
// touch main-region slots already read or free.
#pragma once
#include "cpic_common.cuh"
#include "cpic_bits.h"

namespace cpic {

// =================================================================== F64

struct F64 {
	struct Rec { double x, y, ux, uy; int32_t id; };
	static constexpr int kMinBlocks = 1;

	struct Out {
		int dest;        // destination tile
		int rx, ry;      // new cell relative to the tile origin (unwrapped)
		long long w[4];  // fixed-point deposit w00, w01, w10, w11 (high word)
		long long wl[4]; // remainder words, 2^m finer
		int quirk;       // position exactly on the upper boundary
		int qx, qy;      // quirk: raw node indices
		uint32_t err;
	};

	// shared memory: W x W 64-bit high words, then W x W remainder words
	static __host__ __device__ size_t smem_bytes(int W, int T)
	{
		return 2 * (size_t) W * W * sizeof(long long);
	}

	static __device__ __forceinline__ Rec load(const PushArgs &a, int s, int64_t i)
	{
		const StoreF64 &st = a.f64[s];
		Rec r;
		r.x = st.x[i]; r.y = st.y[i]; r.ux = st.ux[i]; r.uy = st.uy[i];
		r.id = st.id[i];
		return r;
	}

	static __device__ __forceinline__ void store(const PushArgs &a, int s, int64_t i, const Rec &r)
	{
		const StoreF64 &st = a.f64[s];
		st.x[i] = r.x; st.y[i] = r.y; st.ux[i] = r.ux; st.uy[i] = r.uy;
		st.id[i] = r.id;
	}

	// the FP64 store always keeps ids
	template <bool kIds>
	static __device__ __forceinline__ void store_t(const PushArgs &a, int s, int64_t i, const Rec &r)
	{
		store(a, s, i, r);
	}

	// Staged chunk layout: x, y, ux, uy (C doubles each), id, for a chunk
	// of C particles.
	static __host__ __device__ __forceinline__ size_t stage_bytes(bool, int C)
	{
		return (size_t) C * (4 * sizeof(double) + sizeof(int32_t));
	}

	// Thread 0: arm `bar` and copy particles [c0, c0 + cnt) of the tile.
	template <int C>
	static __device__ __forceinline__ void stage_issue(const PushArgs &a, int s, int64_t first,
			int cnt, unsigned char *buf, uint64_t *bar)
	{
		const StoreF64 &st = a.f64[s];
		uint32_t b8 = (uint32_t) ((cnt * 8 + 15) & ~15);
		uint32_t b4 = (uint32_t) ((cnt * 4 + 15) & ~15);
		mbar_arrive_expect_tx(bar, 4 * b8 + b4);
		bulk_g2s(buf, st.x + first, b8, bar);
		bulk_g2s(buf + C * 8, st.y + first, b8, bar);
		bulk_g2s(buf + C * 16, st.ux + first, b8, bar);
		bulk_g2s(buf + C * 24, st.uy + first, b8, bar);
		bulk_g2s(buf + C * 32, st.id + first, b4, bar);
	}

	template <int C>
	static __device__ __forceinline__ Rec from_stage(const unsigned char *buf, int j, bool)
	{
		const double *d = reinterpret_cast<const double *>(buf);
		Rec r;
		r.x = d[j]; r.y = d[C + j]; r.ux = d[2 * C + j]; r.uy = d[3 * C + j];
		r.id = reinterpret_cast<const int32_t *>(buf + C * 32)[j];
		return r;
	}

	// relative_position_grid, interpolate.c:38-66 (field origin 0 on one
	// rank).  The cell index is floor() converted to int, as
	// vf64_to_vi64 does for in-range values (simd_avx2.h:238-248).
	// The floor and its conversion to int are done on the integer pipe
	// (cpic_bits.h, exact) for positions in the box, the FP64 instructions
	// otherwise.
	static __device__ __forceinline__ double rel_pos(double x, double dx, double idx, int &i0)
	{
		double block_delta = x - 0.0;
		double block_rel = block_delta * idx;
		double block_start;
		if(!bits::floor_nonneg(block_rel, block_start, i0))
		{
			block_start = floor(block_rel);
			i0 = (int) block_start;
		}
		double grid_delta = block_delta - block_start * dx;
		return grid_delta * idx;
	}

	// weights(), interpolate.c:77-100 (Y uses dx[X], interpolate.c:88)
	// and linear_interpolation, interpolate.c:11-32.
	static __device__ __forceinline__ void weights(const Grid &g, double x, double y,
			double w[4], int &i0x, int &i0y)
	{
		double rx = rel_pos(x, g.dx, g.idx, i0x);
		double ry = rel_pos(y, g.dx, g.idy, i0y);
		double delx = 1.0 - rx, dely = 1.0 - ry;
		w[0] = delx * dely;
		w[1] = delx * ry;
		w[2] = rx * dely;
		w[3] = rx * ry;
	}

	// interpolate_f2p, interpolate.c:102-155: nodes (i0x,i0y) (i0x,i1y)
	// (i1x,i0y) (i1x,i1y) in that order; i1x wraps, i1y is the ghost row.
	// Index = iy * nx + ix exactly as MAT_XY on E (real_shape[X] = nx).
	static __device__ __forceinline__ void gather(const double *Ex, const double *Ey,
			const Grid &g, const double w[4], int i0x, int i0y, double &ex, double &ey)
	{
		int64_t nx = g.nx;
		int i1x = i0x + 1, i1y = i0y + 1;
		if(i1x >= g.nx) i1x -= g.nx;
		int64_t n00 = (int64_t) i0y * nx + i0x, n01 = (int64_t) i1y * nx + i0x;
		int64_t n10 = (int64_t) i0y * nx + i1x, n11 = (int64_t) i1y * nx + i1x;
		double v;
		v  = w[0] * Ex[n00];
		v += w[1] * Ex[n01];
		v += w[2] * Ex[n10];
		v += w[3] * Ex[n11];
		ex = v;
		v  = w[0] * Ey[n00];
		v += w[1] * Ey[n01];
		v += w[2] * Ey[n10];
		v += w[3] * Ey[n11];
		ey = v;
	}

	// One particle.  tx0/ty0: origin of the tile it is processed in.
	// deposit_only: keep the state, only compute the deposit (pre-step).
	template <bool GP2 = true>
	static __device__ __forceinline__ Out push(const PushArgs &a, int s, Rec &r,
			int tx0, int ty0, const void *)
	{
		const Grid &g = a.g;
		const SpeciesStep &sp = a.sp[s];
		Out o;
		o.err = 0;
		o.quirk = 0;
		double w[4];
		int i0x, i0y;
		weights(g, r.x, r.y, w, i0x, i0y);
		if(i0x < 0 || i0y < 0 || i0x > g.nx || i0y > g.ny)
		{
			o.err |= ST_RANGE;
			i0x = min(max(i0x, 0), g.nx - 1);
			i0y = min(max(i0y, 0), g.ny - 1);
		}
		double ex, ey;
		gather(a.Ex64, a.Ey64, g, w, i0x, i0y, ex, ey);

		// boris_rotation, mover.c:22-70, with B = (0, 0, Bz): the terms
		// multiplied by the exact zeros t[X], t[Y], s[X], s[Y] vanish
		// exactly, leaving these operations in the same order.
		double dtqm2 = sp.dtqm2;
		double vmx = r.ux + dtqm2 * ex;
		double vmy = r.uy + dtqm2 * ey;
		double vpx = vmy * sp.tz + vmx;
		double vpy = vmy - vmx * sp.tz;
		double vlx = vpy * sp.sz + vmx;
		double vly = vmy - vpx * sp.sz;
		double ux = vlx + dtqm2 * ex;
		double uy = vly + dtqm2 * ey;

		// check_velocity, mover.c:97-137 (the compares on the integer
		// pipe, cpic_bits.h: the same results)
		if(bits::abs_gt(ux, sp.umax_x) || bits::abs_gt(uy, sp.umax_y))
			o.err |= ST_UMAX;
		if(!bits::is_finite(ux) || !bits::is_finite(uy))
			o.err |= ST_NAN;

		double x = r.x, y = r.y;
		if(a.iter != 0)
		{
			// move, mover.c:74-82
			x += ux * a.dt;
			y += uy * a.dt;
		}
		// periodic_boundary_ppack, comm_plasma.c:725-747 (X then Y; the
		// compares on the integer pipe, cpic_bits.h).  A branch around the
		// rare wrap: computed for every particle and selected, the two
		// additions took 4 % of the FP64 form's time.
		if(__builtin_expect(bits::ge_pos(x, g.Lx) || bits::lt_zero(x), 0))
			x = bits::ge_pos(x, g.Lx) ? x - g.Lx : x + g.Lx;
		if(__builtin_expect(bits::ge_pos(y, g.Ly) || bits::lt_zero(y), 0))
			y = bits::ge_pos(y, g.Ly) ? y - g.Ly : y + g.Ly;
		if(!bits::is_finite(x) || !bits::is_finite(y))
		{
			o.err |= ST_NAN;
			x = 0.0; y = 0.0;
		}
		r.x = x; r.y = y; r.ux = ux; r.uy = uy;

		// deposit weights of the new position (interpolate_p2f,
		// interpolate.c:161-276), value w * (-q/e0) in two-word fixed
		// point: c = w * qfix is the reference's addend scaled by 2^k
		// (exactly: a power-of-two scale), hi its rounding, and the
		// remainder c - hi (exact) is kept at 2^m finer resolution.
		weights(g, x, y, w, i0x, i0y);
		for(int c = 0; c < 4; c++)
		{
			double v = w[c] * sp.qfix;
			// the split on the integer pipe (cpic_bits.h: exact, the same
			// values), the FP64 instructions for what it does not take
			long long hi, lo;
			if(!bits::split_fixed(v, sp.qlo_exp, hi, lo))
			{
				hi = __double2ll_rn(v);
				lo = __double2ll_rn((v - (double) hi) * sp.qlo_mul);
			}
			o.w[c] = hi;
			o.wl[c] = lo;
		}
		if(i0x >= g.nx || i0y >= g.ny || i0x < 0 || i0y < 0)
		{
			// x == L or y == L after the wrap: keep the reference's
			// node indices (column nx is FFT padding, row ny+1 is
			// outside rho).
			o.quirk = 1;
			o.qx = i0x; o.qy = i0y;
			int cx = min(max(i0x, 0), g.nx - 1), cy = min(max(i0y, 0), g.ny - 1);
			o.dest = tile_of(g, cx, cy);
			o.rx = 0; o.ry = 0;
			return o;
		}
		o.dest = tile_of(g, i0x, i0y);
		int rx = i0x - tx0, ry = i0y - ty0;
		if(rx > g.nx / 2) rx -= g.nx;
		else if(rx < -g.nx / 2) rx += g.nx;
		if(ry > g.ny / 2) ry -= g.ny;
		else if(ry < -g.ny / 2) ry += g.ny;
		o.rx = rx; o.ry = ry;
		return o;
	}

	static __device__ __forceinline__ void clear(unsigned char *sm, int W, int T)
	{
		long long *acc = reinterpret_cast<long long *>(sm);
		for(int i = threadIdx.x; i < 2 * W * W; i += blockDim.x)
			acc[i] = 0;
	}

	static __device__ __forceinline__ int near_full(unsigned char *, int, int) { return 0; }
	static __device__ __forceinline__ void fold(const PushArgs &, int, unsigned char *, int, int,
			int, int) {}

	// Deposit into the tile accumulator, or globally outside the halo, or
	// with the reference's node indices for the boundary quirk
	// (contributions to column nx, the FFT padding, and row ny+1 are
	// dropped; row ny folds into row 0).
	static __device__ __forceinline__ void deposit(const PushArgs &a, int s, unsigned char *sm,
			int W, int H, int tx0, int ty0, const Out &o)
	{
		const Grid &g = a.g;
		if(o.quirk)
		{
			int i0x = o.qx, i0y = o.qy;
			int i1x = i0x + 1; if(i1x >= g.nx) i1x -= g.nx;
			int i1y = i0y + 1;
			int xs[4] = {i0x, i0x, i1x, i1x};
			int ys[4] = {i0y, i1y, i0y, i1y};
			for(int c = 0; c < 4; c++)
			{
				int x = xs[c], y = ys[c];
				if(x < 0 || x >= g.nx || y < 0 || y > g.ny) continue;
				if(y == g.ny) y = 0;
				red_global(&a.rho[(int64_t) y * g.nx + x], o.w[c]);
				red_global(&a.rho_lo[(int64_t) y * g.nx + x], o.wl[c]);
			}
			return;
		}
		int lx = o.rx + H, ly = o.ry + H;
		if(sm && (unsigned) lx < (unsigned) (W - 1) && (unsigned) ly < (unsigned) (W - 1))
		{
			long long *p = reinterpret_cast<long long *>(sm) + ly * W + lx;
			long long *q = p + W * W;
			atomicAdd((unsigned long long *) &p[0], (unsigned long long) o.w[0]);
			atomicAdd((unsigned long long *) &p[W], (unsigned long long) o.w[1]);
			atomicAdd((unsigned long long *) &p[1], (unsigned long long) o.w[2]);
			atomicAdd((unsigned long long *) &p[W + 1], (unsigned long long) o.w[3]);
			atomicAdd((unsigned long long *) &q[0], (unsigned long long) o.wl[0]);
			atomicAdd((unsigned long long *) &q[W], (unsigned long long) o.wl[1]);
			atomicAdd((unsigned long long *) &q[1], (unsigned long long) o.wl[2]);
			atomicAdd((unsigned long long *) &q[W + 1], (unsigned long long) o.wl[3]);
		}
		else
			dep_global2(a.rho, a.rho_lo, g, tx0 + o.rx, ty0 + o.ry, o.w, o.wl);
	}

	static __device__ __forceinline__ void flush(const PushArgs &a, int s, unsigned char *sm,
			int W, int H, int tx0, int ty0)
	{
		const long long *acc = reinterpret_cast<const long long *>(sm);
		for(int i = threadIdx.x; i < W * W; i += blockDim.x)
		{
			long long v = acc[i], vl = acc[W * W + i];
			int64_t node = frame_node(a.g, W, H, tx0, ty0, i);
			if(v != 0) red_global(&a.rho[node], v);
			if(vl != 0) red_global(&a.rho_lo[node], vl);
		}
	}

	static __device__ __forceinline__ const void *load_field(const PushArgs &, unsigned char *,
			int, int, int, int)
	{
		return nullptr;
	}

	// the FP64 form reads E from global memory: no field tile to copy
	static __device__ __forceinline__ bool field_tma(const PushArgs &, int, int) { return false; }
	static __device__ __forceinline__ const void *field_tile(unsigned char *) { return nullptr; }
	static __device__ __forceinline__ const void *field_issue(const PushArgs &, unsigned char *,
			int, int, uint64_t *)
	{
		return nullptr;
	}

	static __device__ __forceinline__ Rec from_spill(const Spill &S, int64_t k, const Grid &)
	{
		Rec r;
		r.x = S.x[k]; r.y = S.y[k]; r.ux = S.ux[k]; r.uy = S.uy[k]; r.id = S.id[k];
		return r;
	}

	static __device__ __forceinline__ void to_spill_vals(const Rec &r, const Grid &,
			double &x, double &y, double &ux, double &uy)
	{
		x = r.x; y = r.y; ux = r.ux; uy = r.uy;
	}

	static __device__ __forceinline__ void to_spill_rec(const Rec &r, const Grid &g,
			double &x, double &y, double &ux, double &uy)
	{
		to_spill_vals(r, g, x, y, ux, uy);
	}

	static __device__ __forceinline__ int cell_of(const Rec &r, const Grid &g, int &cx, int &cy)
	{
		double w[4];
		weights(g, r.x, r.y, w, cx, cy);
		return 0;
	}
};

// =================================================================== Mix

struct Mix {
	struct Rec { int32_t cell; float ox, oy, ux, uy; int32_t id; };
#ifdef CPIC_PUSH_MIN_BLOCKS
	static constexpr int kMinBlocks = CPIC_PUSH_MIN_BLOCKS;
	static constexpr int kHiBlocks = CPIC_PUSH_MIN_BLOCKS;
#else
	static constexpr int kMinBlocks = kPushThreads >= 1024 ? 1 : 1024 / kPushThreads;
	// second instance, registers capped for 48 resident warps per SM: used
	// when that many blocks fit in shared memory
	static constexpr int kHiBlocks = kPushThreads >= 1536 ? 1 : 1536 / kPushThreads;
#endif

	struct Out {
		int dest;
		int rx, ry;
		uint32_t wq[4];  // weights round(w * 2^kWeightBits)
		uint32_t err;
	};

	// shared memory: the E tile, T + 1 rows of T + 1 nodes with a row
	// pitch of T + 2 (the tensor copy's box is an even number of 8-byte
	// elements wide), then the W x W u32 accumulator
	static __host__ __device__ size_t smem_bytes(int W, int T)
	{
		return (size_t) W * W * sizeof(uint32_t) + (size_t) (T + 2) * (T + 1) * sizeof(float2);
	}

	static __device__ __forceinline__ Rec load(const PushArgs &a, int s, int64_t i)
	{
		const StoreMix &st = a.mix[s];
		Rec r;
		r.cell = st.cell[i];
		const float4 v = st.ou[i];
		r.ox = v.x; r.oy = v.y; r.ux = v.z; r.uy = v.w;
		r.id = st.id ? st.id[i] : 0;
		return r;
	}

	static __device__ __forceinline__ void store(const PushArgs &a, int s, int64_t i, const Rec &r)
	{
		const StoreMix &st = a.mix[s];
		st.cell[i] = r.cell;
		st.ou[i] = make_float4(r.ox, r.oy, r.ux, r.uy);
		if(st.id) st.id[i] = r.id;
	}

	// kIds: whether the store keeps ids, known at compile time (no branch
	// in the fused kernel's write-back)
	template <bool kIds>
	static __device__ __forceinline__ void store_t(const PushArgs &a, int s, int64_t i, const Rec &r)
	{
		const StoreMix &st = a.mix[s];
		st.cell[i] = r.cell;
		st.ou[i] = make_float4(r.ox, r.oy, r.ux, r.uy);
		if(kIds) st.id[i] = r.id;
	}

	// Staged chunk layout: cell (C 32-bit words), the (ox, oy, ux, uy)
	// quadruples (C x 16 bytes) and, when ids are tracked, id, for a chunk
	// of C particles.
	static __host__ __device__ __forceinline__ size_t stage_bytes(bool ids, int C)
	{
		return (size_t) C * 4 * (ids ? 6 : 5);
	}

	template <int C>
	static __device__ __forceinline__ void stage_issue(const PushArgs &a, int s, int64_t first,
			int cnt, unsigned char *buf, uint64_t *bar)
	{
		const StoreMix &st = a.mix[s];
		uint32_t b4 = (uint32_t) ((cnt * 4 + 15) & ~15);
		uint32_t b16 = (uint32_t) cnt * 16;
		mbar_arrive_expect_tx(bar, (st.id ? 2 : 1) * b4 + b16);
		bulk_g2s(buf, st.cell + first, b4, bar);
		bulk_g2s(buf + C * 4, st.ou + first, b16, bar);
		if(st.id)
			bulk_g2s(buf + C * 20, st.id + first, b4, bar);
	}

	template <int C>
	static __device__ __forceinline__ Rec from_stage(const unsigned char *buf, int j, bool ids)
	{
		Rec r;
		r.cell = reinterpret_cast<const int32_t *>(buf)[j];
		const float4 v = reinterpret_cast<const float4 *>(buf + C * 4)[j];
		r.ox = v.x; r.oy = v.y; r.ux = v.z; r.uy = v.w;
		r.id = ids ? reinterpret_cast<const int32_t *>(buf)[5 * C + j] : 0;
		return r;
	}

	// round(w * 2^kWeightBits) for w in [0, 1]: adding 2^23 puts the
	// rounded integer in the low mantissa bits.
	static __device__ __forceinline__ uint32_t wfix(float w)
	{
		float f = __fmaf_rn(w, (float) (1 << kWeightBits), 8388608.0f);
		return __float_as_uint(f) - 0x4B000000u;
	}

	// Etile: shared tile of E at the tile's (T+1) x (T+1) nodes (row pitch
	// T + 2), or null for the global field (spill records).
	template <bool GP2 = true>
	static __device__ __forceinline__ Out push(const PushArgs &a, int s, Rec &r,
			int tx0, int ty0, const void *Etile)
	{
		const Grid &g = a.g;
		const SpeciesStep &sp = a.sp[s];
		Out o;
		o.err = 0;
		// Every floating-point operation below is an explicit-rounding
		// intrinsic: the fused kernel and the spill pass compile this
		// function separately, and the compiler may not contract or
		// reassociate differently in the two, so a particle gets the same
		// result on either path.
		int cx = r.cell & ((1 << g.lcx) - 1), cy = r.cell >> g.lcx;
		float ox = r.ox, oy = r.oy;
		float dxo = __fsub_rn(1.0f, ox), dyo = __fsub_rn(1.0f, oy);
		float w00 = __fmul_rn(dxo, dyo), w01 = __fmul_rn(dxo, oy);
		float w10 = __fmul_rn(ox, dyo), w11 = __fmul_rn(ox, oy);
		float2 e00, e01, e10, e11;
		const int lx = cx - tx0, ly = cy - ty0;
		if(Etile && (unsigned) lx < (unsigned) g.tx && (unsigned) ly < (unsigned) g.ty)
		{
			const float2 *Et = (const float2 *) Etile;
			int W = g.tx + 2;
			const float2 *p = Et + ly * W + lx;
			e00 = p[0]; e01 = p[W]; e10 = p[1]; e11 = p[W + 1];
		}
		else
		{
			// spill records, and particles kept outside their tile when
			// their destination and the spill list were both full
			int x1 = wrapn(cx + 1, g.nx), y1 = wrapn(cy + 1, g.ny);
			e00 = a.E32[(int64_t) cy * g.nx + cx];
			e01 = a.E32[(int64_t) y1 * g.nx + cx];
			e10 = a.E32[(int64_t) cy * g.nx + x1];
			e11 = a.E32[(int64_t) y1 * g.nx + x1];
		}
		float ex = __fmaf_rn(w11, e11.x, __fmaf_rn(w10, e10.x, __fmaf_rn(w01, e01.x,
				__fmul_rn(w00, e00.x))));
		float ey = __fmaf_rn(w11, e11.y, __fmaf_rn(w10, e10.y, __fmaf_rn(w01, e01.y,
				__fmul_rn(w00, e00.y))));

		// Boris with B along z (same structure as the FP64 form)
		float dtqm2 = sp.dtqm2_f;
		float hx = __fmul_rn(dtqm2, ex), hy = __fmul_rn(dtqm2, ey);
		float vmx = __fadd_rn(r.ux, hx);
		float vmy = __fadd_rn(r.uy, hy);
		float vpx = __fmaf_rn(vmy, sp.tz_f, vmx);
		float vpy = __fmaf_rn(-vmx, sp.tz_f, vmy);
		float ux = __fadd_rn(__fmaf_rn(vpy, sp.sz_f, vmx), hx);
		float uy = __fadd_rn(__fmaf_rn(-vpx, sp.sz_f, vmy), hy);
		// one compare per component on the common path: a NaN fails
		// |u| <= umax as an out-of-range speed does (0.9 % of the kernel's
		// time against four compares)
		if(!(fabsf(ux) <= sp.umax_x_f) || !(fabsf(uy) <= sp.umax_y_f))
		{
			if(fabsf(ux) > sp.umax_x_f || fabsf(uy) > sp.umax_y_f)
				o.err |= ST_UMAX;
			if(!isfinite(ux) || !isfinite(uy))
			{
				o.err |= ST_NAN;
				ux = 0.0f; uy = 0.0f;
			}
		}
		int sx = 0, sy = 0;
		if(a.iter != 0)
		{
			ox = __fmaf_rn(ux, a.cdx_f, ox);
			oy = __fmaf_rn(uy, a.cdy_f, oy);
			float fx = floorf(ox), fy = floorf(oy);
			ox = __fsub_rn(ox, fx); oy = __fsub_rn(oy, fy);
			sx = (int) fx; sy = (int) fy;
			if(ox >= 1.0f) { ox = __fsub_rn(ox, 1.0f); sx += 1; }
			if(oy >= 1.0f) { oy = __fsub_rn(oy, 1.0f); sy += 1; }
		}
		// the new cell, wrapped: a mask on a power-of-two grid; else a
		// compare, and a division only for a move beyond one period (a
		// particle over the velocity limit, already flagged)
		int ncx = cx + sx, ncy = cy + sy;
		if(GP2)
		{
			ncx = wrap2(ncx, g.nx);
			ncy = wrap2(ncy, g.ny);
		}
		else
		{
			if((unsigned) ncx >= (unsigned) g.nx) ncx = wrap_mod(ncx, g.nx);
			if((unsigned) ncy >= (unsigned) g.ny) ncy = wrap_mod(ncy, g.ny);
		}
		r.cell = (ncy << g.lcx) + ncx;
		r.ox = ox; r.oy = oy; r.ux = ux; r.uy = uy;

		dxo = __fsub_rn(1.0f, ox); dyo = __fsub_rn(1.0f, oy);
		o.wq[0] = wfix(__fmul_rn(dxo, dyo));
		o.wq[1] = wfix(__fmul_rn(dxo, oy));
		o.wq[2] = wfix(__fmul_rn(ox, dyo));
		o.wq[3] = wfix(__fmul_rn(ox, oy));
		o.dest = tile_of(g, ncx, ncy);
		if(Etile)
		{
			o.rx = cx - tx0 + sx;
			o.ry = cy - ty0 + sy;
		}
		else
		{
			o.rx = ncx - tx0;
			o.ry = ncy - ty0;
		}
		return o;
	}

	// Shared layout: [float2 E tile (T+1) x (T+2)][u32 accumulator W*W].
	static __device__ __forceinline__ float2 *shE(unsigned char *sm, int)
	{
		return reinterpret_cast<float2 *>(sm);
	}
	static __device__ __forceinline__ uint32_t *sh32(unsigned char *sm, int, int T)
	{
		return reinterpret_cast<uint32_t *>(sm + (size_t) (T + 2) * (T + 1) * 8);
	}

	static __device__ __forceinline__ void clear(unsigned char *sm, int W, int T)
	{
		uint32_t *a32 = sh32(sm, W, T);
		for(int i = threadIdx.x; i < W * W; i += blockDim.x)
			a32[i] = 0;
	}

	// Some node's sum has reached 2^30 (this thread's share of the nodes).
	static __device__ __forceinline__ int near_full(unsigned char *sm, int W, int T)
	{
		const uint32_t *a32 = sh32(sm, W, T);
		uint32_t m = 0;
		for(int i = threadIdx.x; i < W * W; i += blockDim.x)
			m |= a32[i];
		return (m >> 30) != 0;
	}

	// Fixed-point units of v integer weight units: an integer product when
	// the species' factor is an exact integer (then (double) v * sc is exact
	// too, so both give the same value; the integer one keeps the FP64 pipe,
	// narrow on this GPU, out of the fold and flush; the per-particle global
	// fallback keeps the FP64 form, which needs fewer registers inside the
	// particle loop).
	static __device__ __forceinline__ long long wunits(uint32_t v, const SpeciesStep &sp)
	{
		return sp.wq_int ? (long long) v * sp.wq_int : __double2ll_rn((double) v * sp.wq_scale);
	}

	// Add the 32-bit sums to global rho and restart them from zero
	// (between barriers).  With the species' fixed-point factor an exact
	// integer, the partial sums add up to exactly the value one flush of
	// the whole tile gives.
	static __device__ __forceinline__ void fold(const PushArgs &a, int s, unsigned char *sm,
			int W, int H, int tx0, int ty0)
	{
		uint32_t *a32 = sh32(sm, W, a.g.tx);
		const SpeciesStep &sp = a.sp[s];
		for(int i = threadIdx.x; i < W * W; i += blockDim.x)
		{
			uint32_t v = a32[i];
			if(v != 0)
			{
				red_global(&a.rho[frame_node(a.g, W, H, tx0, ty0, i)], wunits(v, sp));
				a32[i] = 0;
			}
		}
	}

	static __device__ __forceinline__ void deposit(const PushArgs &a, int s, unsigned char *sm,
			int W, int H, int tx0, int ty0, const Out &o)
	{
		int lx = o.rx + H, ly = o.ry + H;
		if(sm && (unsigned) lx < (unsigned) (W - 1) && (unsigned) ly < (unsigned) (W - 1))
		{
			uint32_t *p = sh32(sm, W, a.g.tx) + ly * W + lx;
			atomicAdd(&p[0], o.wq[0]);
			atomicAdd(&p[W], o.wq[1]);
			atomicAdd(&p[1], o.wq[2]);
			atomicAdd(&p[W + 1], o.wq[3]);
		}
		else
		{
			double sc = a.sp[s].wq_scale;
			dep_global(a.rho, a.g, tx0 + o.rx, ty0 + o.ry,
					__double2ll_rn((double) o.wq[0] * sc), __double2ll_rn((double) o.wq[1] * sc),
					__double2ll_rn((double) o.wq[2] * sc), __double2ll_rn((double) o.wq[3] * sc));
		}
	}

	static __device__ __forceinline__ void flush(const PushArgs &a, int s, unsigned char *sm,
			int W, int H, int tx0, int ty0)
	{
		const uint32_t *a32 = sh32(sm, W, a.g.tx);
		const SpeciesStep &sp = a.sp[s];
		for(int i = threadIdx.x; i < W * W; i += blockDim.x)
		{
			uint32_t v = a32[i];
			if(v != 0)
				red_global(&a.rho[frame_node(a.g, W, H, tx0, ty0, i)], wunits(v, sp));
		}
	}

	// The field tile by per-thread loads (nodes past the grid's last row
	// or column wrap to the first).
	static __device__ __forceinline__ const void *load_field(const PushArgs &a, unsigned char *sm,
			int W, int T, int tx0, int ty0)
	{
		const Grid &g = a.g;
		float2 *Et = shE(sm, W);
		const int WE = g.tx + 1;
		for(int i = threadIdx.x; i < WE * (g.ty + 1); i += blockDim.x)
		{
			int lx = i % WE, ly = i / WE;
			int gx = wrapn(tx0 + lx, g.nx), gy = wrapn(ty0 + ly, g.ny);
			Et[ly * (g.tx + 2) + lx] = a.E32[(int64_t) gy * g.nx + gx];
		}
		return Et;
	}

	// Whether this tile's field comes by one 2D tensor copy: a map exists
	// (tiles of an even width, so the box starts on a 16-byte boundary)
	// and the tile is not in the grid's last column or row, whose nodes
	// wrap (those tiles load by threads).  The box's extra column is read
	// and never used.
	static __device__ __forceinline__ bool field_tma(const PushArgs &a, int tx0, int ty0)
	{
		return a.emap_ok && tx0 + a.g.tx < a.g.nx && ty0 + a.g.ty < a.g.ny;
	}

	static __device__ __forceinline__ const void *field_tile(unsigned char *sm)
	{
		return shE(sm, 0);
	}

	// Thread 0: arm bar with the box's bytes and copy the tile's field.
	static __device__ __forceinline__ const void *field_issue(const PushArgs &a, unsigned char *sm,
			int tx0, int ty0, uint64_t *bar)
	{
		float2 *Et = shE(sm, 0);
		mbar_arrive_expect_tx(bar, (uint32_t) ((a.g.tx + 2) * (a.g.ty + 1) * sizeof(float2)));
		tensor_g2s_2d(Et, &a.emap, tx0, ty0, bar);
		return Et;
	}

	static __device__ __forceinline__ Rec from_spill(const Spill &S, int64_t k, const Grid &g)
	{
		Rec r;
		double px = S.cell_units ? S.x[k] : S.x[k] * g.idx;
		double py = S.cell_units ? S.y[k] : S.y[k] * g.idy;
		double fx = floor(px), fy = floor(py);
		int cx = wrap_mod((int) fx, g.nx), cy = wrap_mod((int) fy, g.ny);
		float ox = (float) (px - fx), oy = (float) (py - fy);
		if(ox >= 1.0f) { ox = 0.0f; cx = wrapn(cx + 1, g.nx); }
		if(oy >= 1.0f) { oy = 0.0f; cy = wrapn(cy + 1, g.ny); }
		r.cell = (cy << g.lcx) + cx;
		r.ox = ox; r.oy = oy;
		r.ux = (float) S.ux[k]; r.uy = (float) S.uy[k];
		r.id = S.id[k];
		return r;
	}

	static __device__ __forceinline__ void to_spill_vals(const Rec &r, const Grid &g,
			double &x, double &y, double &ux, double &uy)
	{
		int cx = r.cell & ((1 << g.lcx) - 1), cy = r.cell >> g.lcx;
		x = ((double) cx + (double) r.ox) * g.dx;
		y = ((double) cy + (double) r.oy) * g.dy;
		ux = r.ux; uy = r.uy;
	}

	// A spill record in cell units (cell_units lists): cx + ox is exact in
	// FP64, so a record that passes through the spill list is unchanged.
	static __device__ __forceinline__ void to_spill_rec(const Rec &r, const Grid &g,
			double &x, double &y, double &ux, double &uy)
	{
		int cx = r.cell & ((1 << g.lcx) - 1), cy = r.cell >> g.lcx;
		x = (double) cx + (double) r.ox;
		y = (double) cy + (double) r.oy;
		ux = r.ux; uy = r.uy;
	}

	static __device__ __forceinline__ int cell_of(const Rec &r, const Grid &g, int &cx, int &cy)
	{
		cx = r.cell & ((1 << g.lcx) - 1);
		cy = r.cell >> g.lcx;
		return 0;
	}
};

// ============================================================== kernels

// Ids: whether the species' store keeps particle ids (always for F64).
// P: particles per thread per chunk (a chunk is kPushThreads * P particles).
// GP2: nx and ny are powers of two (the mixed form wraps cells with a mask).
template <class F, int MinBlocks = F::kMinBlocks, bool Ids = true, int P = kPPT, bool GP2 = true>
__global__ void __launch_bounds__(kPushThreads, MinBlocks)
k_push(const __grid_constant__ PushArgs a)
{
	constexpr int kChunk = chunk_of(P);
	constexpr int kCheckChunks = check_chunks(P);
	// dynamic shared memory: two staged chunks, then the form's area
	extern __shared__ __align__(128) unsigned char smem[];
	__shared__ __align__(8) uint64_t bars[2];
	__shared__ __align__(8) uint64_t ebars[2];
	__shared__ __align__(8) uint64_t fbar;   // the field tile's tensor copy
	__shared__ int s_cursor;
	__shared__ int s_timeout;        // a bounded wait of this block expired
	// arrivals base (in the buffer this step writes) and capacity of the
	// 3 x 3 tiles around this one: nearly every mover lands there, so its
	// slot needs no dependent global loads
	__shared__ int64_t s_nbase[9];
	__shared__ int32_t s_ncap[9];
	const Grid &g = a.g;
	// one launch per species, its data at index 0: every parameter access
	// has a fixed offset (no indexed constant loads in the particle loop)
	const int s = 0;
	const Tiles &T = a.tiles[s];
	// blocks are dispatched in index order; the order array puts the
	// heaviest tiles first (a permutation, so every tile is taken once)
	const int t = T.order ? T.order[blockIdx.x] : (int) blockIdx.x;
	if((unsigned) t >= gridDim.x)
	{
		if(threadIdx.x == 0) set_status(a.status, ST_RANGE);
		return;
	}
	const int H = g.halo;
	const int W = g.tx + 2 * H + 1;
	int ttx, tty;
	tile_rc(g, t, ttx, tty);
	const int tx0 = ttx << g.ltx;
	const int ty0 = tty << g.lty;
	const bool ids = Ids;
	const size_t sb = F::stage_bytes(ids, kChunk);
	// bulk-copy destinations need 16-byte alignment; the host adds 128
	// bytes of slack for this round-up.  An offset from smem (not a pointer
	// rebuilt from an integer) keeps every derived pointer in the shared
	// space, so accesses compile to shared-memory loads and atomics.
	unsigned char *stage0 = smem
		+ ((128u - (unsigned) (reinterpret_cast<uintptr_t>(smem) & 127u)) & 127u);
	unsigned char *fsm = stage0 + 2 * sb;

	F::clear(fsm, W, g.tx);
	// the field tile: one 2D tensor copy (issued with the barriers below)
	// where the form has a map for it, else per-thread loads
	const bool ftma = F::field_tma(a, tx0, ty0);
	const void *Etile = ftma ? F::field_tile(fsm) : F::load_field(a, fsm, W, g.tx, tx0, ty0);
	// the chunks: the main region's particles, then the arrivals the
	// previous step left in buffer r; a chunk never spans both, so every
	// bulk copy starts on a 32-slot boundary
	const int r = a.arr_r;
	const int nm = T.cnt[t];
	// (a count can pass the capacity: movers that found the region full
	// went to the spill list but still took a slot number)
	const int na = min(T.acnt[r][t], T.acap[t]);
	const int64_t base = T.base[t];
	const int capt = T.cap[t];
	const int64_t abase_r = T.abase[t] + (r ? T.abuf1 : 0);
	const int64_t aofs_w = r ? 0 : T.abuf1;
	int32_t *const acnt_w = T.acnt[r ^ 1];
	const int nmc = (nm + kChunk - 1) / kChunk;
	const int nchunks = nmc + (na + kChunk - 1) / kChunk;
	auto chunk = [&](int ci, int64_t &first, int &len) {
		if(ci < nmc)
		{
			first = base + (int64_t) ci * kChunk;
			len = min(kChunk, nm - ci * kChunk);
		}
		else
		{
			const int o = (ci - nmc) * kChunk;
			first = abase_r + o;
			len = min(kChunk, na - o);
		}
	};
	// neighbours are distinct tiles only with at least 3 tiles per side
	const bool nb_ok = g.ntx >= 3 && g.nty >= 3;
	if(threadIdx.x < 9 && nb_ok)
	{
		int dx = (int) threadIdx.x % 3 - 1, dy = (int) threadIdx.x / 3 - 1;
		int nt = wrapn(tty + dy, g.nty) * g.ntx + wrapn(ttx + dx, g.ntx);
		s_nbase[threadIdx.x] = T.abase[nt] + aofs_w;
		s_ncap[threadIdx.x] = T.acap[nt];
	}
	if(threadIdx.x == 0)
	{
		s_cursor = 0;
		s_timeout = 0;
		mbar_init(&bars[0], 1);          // "full": one arrival + bytes
		mbar_init(&bars[1], 1);
		mbar_init(&ebars[0], kPushThreads / 32);   // "empty": one per warp
		mbar_init(&ebars[1], kPushThreads / 32);
		mbar_init(&fbar, 1);
		fence_mbar_init();
		if(ftma)
			F::field_issue(a, fsm, tx0, ty0, &fbar);
	}
	__syncthreads();
	if(threadIdx.x == 0 && nchunks > 0)
	{
		int64_t f0;
		int l0;
		chunk(0, f0, l0);
		F::template stage_issue<kChunk>(a, s, f0, l0, stage0, &bars[0]);
	}
	const int lane = threadIdx.x & 31;
	if(ftma && !mbar_wait_bounded(&fbar, 0, a.status))
		s_timeout = 1;

	for(int ci = 0; ci < nchunks; ci++)
	{
		int64_t cfirst;
		int clen;
		chunk(ci, cfirst, clen);
		if(ci > 0 && ci % kCheckChunks == 0)
		{
			// every deposit of the previous chunks precedes the check (and
			// the fold), and the fold precedes every later deposit.  At
			// typical densities a node's sum over the whole tile stays far
			// below 2^30 and the fold never runs.
			if(__syncthreads_or(F::near_full(fsm, W, g.tx)))
			{
				F::fold(a, s, fsm, W, H, tx0, ty0);
				__syncthreads();
			}
		}
		// prefetch the next chunk into the other buffer once every warp
		// has released it (its last reader was chunk ci - 1)
		if(threadIdx.x == 0 && ci + 1 < nchunks)
		{
			const int b = (ci + 1) & 1;
			if(ci >= 1 && !mbar_wait_bounded(&ebars[b], ((ci - 1) >> 1) & 1, a.status))
				s_timeout = 1;
			fence_proxy_async_smem();
			int64_t nf;
			int nl;
			chunk(ci + 1, nf, nl);
			F::template stage_issue<kChunk>(a, s, nf, nl, stage0 + b * sb, &bars[b]);
		}
		// this chunk has landed: every global read of the main region's
		// slots below the end of this chunk is complete, so the in-place
		// writes below are safe (the stayer cursor never passes the number
		// of particles read; past the main region's count it writes free
		// slots, which nothing reads in this step)
		if(!mbar_wait_bounded(&bars[ci & 1], (ci >> 1) & 1, a.status))
			s_timeout = 1;
		const unsigned char *buf = stage0 + (ci & 1) * sb;
		typename F::Rec rec[P];
		int dest[P];
		unsigned bs[P];
		Resv rv[P];
		uint32_t err = 0;
		#pragma unroll
		for(int k = 0; k < P; k++)
		{
			const int j = k * kPushThreads + threadIdx.x;
			const bool valid = j < clen;
			if(valid)
				rec[k] = F::template from_stage<kChunk>(buf, j, ids);
			// the last record is in registers: this warp is done with the
			// staged chunk, and the buffer goes back to the producer before
			// the last push, not after it (0.7 % faster on the two-stream
			// 2048x2048 benchmark than releasing after the pushes)
			if(k == P - 1)
			{
				__syncwarp();
				if(lane == 0)
					mbar_arrive(&ebars[ci & 1]);
			}
			dest[k] = -1;
			if(valid)
			{
				typename F::Out o = F::template push<GP2>(a, s, rec[k], tx0, ty0, Etile);
				err |= o.err;
				F::deposit(a, s, fsm, W, H, tx0, ty0, o);
				dest[k] = o.dest;
			}
			bs[k] = __ballot_sync(0xffffffffu, dest[k] == t);
			// slots in the destination tiles: atomics issued now, their
			// results consumed after the stayer writes
			rv[k] = warp_reserve_issue(acnt_w, dest[k] >= 0 && dest[k] != t, dest[k]);
		}
		if(err) set_status(a.status, err);
		// one shared-cursor reservation per warp for all its stayers
		int nst = 0;
		#pragma unroll
		for(int k = 0; k < P; k++) nst += __popc(bs[k]);
		int wb = 0;
		if(lane == 0 && nst)
			wb = atomicAdd(&s_cursor, nst);
		wb = __shfl_sync(0xffffffffu, wb, 0);
		// the main region holds this warp's stayers (else, rarely, the
		// ones past its end take the spill list)
		const bool room = wb + nst <= capt;
		// one store per particle: its own tile's compacted prefix, or its
		// slot in the destination tile's arrivals, or the spill list
		#pragma unroll
		for(int k = 0; k < P; k++)
		{
			const bool stay = (bs[k] >> lane) & 1u;
			const bool move = dest[k] >= 0 && dest[k] != t;
			const int slot = warp_reserve_finish(rv[k], move);
			int64_t at = -1;
			bool spill = false;
			if(stay)
			{
				const int idx = wb + __popc(bs[k] & lanemask_lt());
				if(room || idx < capt)
					at = base + idx;
				else
					spill = true;
			}
			else if(move)
			{
				// the neighbour table covers the 3 x 3 tiles around this
				// one; a move across the grid's edge reads the tile's own
				// entries instead (the same values)
				const int d = dest[k];
				int dtx, dty;
				tile_rc(g, d, dtx, dty);
				const int ddx = dtx - ttx + 1;
				const int ddy = dty - tty + 1;
				int64_t db;
				int32_t dc;
				if(nb_ok && (unsigned) ddx < 3u && (unsigned) ddy < 3u)
				{
					db = s_nbase[ddy * 3 + ddx];
					dc = s_ncap[ddy * 3 + ddx];
				}
				else
				{
					db = T.abase[d] + aofs_w;
					dc = T.acap[d];
				}
				if(slot < dc)
					at = db + slot;
				else
					spill = true;
			}
			if(spill)
			{
				double x, y, ux, uy;
				F::to_spill_rec(rec[k], g, x, y, ux, uy);
				// spill list full too: the particle stays in this tile,
				// outside its cell's tile (every later pass handles that),
				// until the host rebuilds the layout; with the main region
				// full as well it is lost, and the status says so
				if(!spill_push(a.spill_out[s], x, y, ux, uy, rec[k].id))
				{
					const int idx = atomicAdd(&s_cursor, 1);
					if(idx < capt)
						at = base + idx;
					else
						set_status(a.status, ST_SPILL_FULL);
				}
			}
			if(at >= 0)
				F::template store_t<Ids>(a, s, at, rec[k]);
			wb += __popc(bs[k]);
		}
	}
	__syncthreads();
	if(threadIdx.x == 0)
	{
		// the main region's count for the next step; this step's arrivals
		// buffer is read and becomes the next step's buffer for movers
		T.cnt[t] = min(s_cursor, capt);
		T.acnt[r][t] = 0;
		// after an expired wait a copy may still be landing in the stage:
		// wait (bounded again) for the last one issued into each buffer
		// before the block's shared memory is released
		if(s_timeout)
		{
			for(int b = 0; b < 2; b++)
			{
				const int c = (nchunks - 1) - (((nchunks - 1) & 1) != b ? 1 : 0);
				if(c >= 0)
					mbar_wait_bounded(&bars[b], (c >> 1) & 1, a.status);
			}
			if(ftma)
				mbar_wait_bounded(&fbar, 0, a.status);
		}
	}
	F::flush(a, s, fsm, W, H, tx0, ty0);
}

// Generic pass over the spill list: records with no tile of their own
// (the particle store overflowed).  E is read from global memory and the
// deposit goes straight to global rho.  Records are placed among their
// tile's arrivals for the next step (the buffer this step's movers go to)
// when it has room, else appended to spill_out.
template <class F>
__global__ void __launch_bounds__(kPushThreads)
k_spill(const SpillArgs sa)
{
	const PushArgs &a = sa.p;
	const Grid &g = a.g;
	for(int s = 0; s < a.nspecies; s++)
	{
		const Spill &S = sa.spill_in[s];
		int ns = *S.count;
		if(ns > S.capacity) ns = S.capacity;
		for(int64_t k0 = (int64_t) blockIdx.x * blockDim.x; k0 < ns;
				k0 += (int64_t) gridDim.x * blockDim.x)
		{
			int64_t k = k0 + threadIdx.x;
			bool valid = k < ns;
			typename F::Rec r;
			typename F::Out o;
			o.dest = 0;
			if(valid)
			{
				r = F::from_spill(S, k, g);
				o = F::template push<false>(a, s, r, 0, 0, nullptr);
				if(o.err) set_status(a.status, o.err);
				F::deposit(a, s, nullptr, 0, 0, 0, 0, o);
			}
			const Tiles &T = a.tiles[s];
			const int w = a.arr_r ^ 1;
			int slot = warp_reserve(T.acnt[w], valid, o.dest);
			if(valid)
			{
				if(slot < T.acap[o.dest])
					F::store(a, s, T.abase[o.dest] + (w ? T.abuf1 : 0) + slot, r);
				else
				{
					double x, y, ux, uy;
					F::to_spill_rec(r, g, x, y, ux, uy);
					// cannot fail: this pass runs first, on an empty
					// list of the same capacity as its input
					if(!spill_push(a.spill_out[s], x, y, ux, uy, r.id))
						set_status(a.status, ST_SPILL_FULL);
				}
			}
		}
	}
}

} // namespace cpic
