/*
 * pp_device.cuh -- device-side building blocks shared by the kernels:
 * Philox4x32-10, uniform integer draws, acquire/release accessors, the run
 * table and the per-world counters.
 *
 * Grass layout: one uint16 per cell holding the run-local iteration at
 * which the cell's grass is (or was) alive again, modulo 2^16; the
 * countdown of iteration t is max(0, (int16)(regrow - t)). Cells are only
 * read where agents are, and written when a sheep eats; the per-iteration
 * grass stats come from a per-run histogram of pending regrowth
 * iterations, updated by the eating events.
 *
 * Agent layout (structure of arrays, one slot per agent):
 *   key[i] = global cell index (y * grid_x + x + run cell base), or the
 *            world's dead sentinel (= number of padded cells) after a move
 *            that killed the agent;
 *   val[i] = type << 31 | energy (the run's energy field width: 11 or
 *            16 bits as the reference's 32- and 64-bit agents, else 30
 *            bits; energy arithmetic is modulo 2^width as there).
 * This replaces the reference's packed agents (pp_gpu.cl:150-316):
 * the cell is the sort key, so the radix sort moves 8 bytes per agent and
 * sorts only ceil(log2(cells + 1)) bits.
 */
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pp {

constexpr uint32_t TYPE_BIT = 0x80000000u;
constexpr uint32_t ENERGY_MASK = 0x7fffffffu;
/* Marks an agent eaten in the act phase's per-agent words, and a newborn
 * in its parent's newborn word (whose energy may be 0): above every energy
 * field width. */
constexpr uint32_t EATEN_BIT = 0x40000000u;
constexpr uint32_t KID_BIT = 0x40000000u;
constexpr uint32_t KID_ENERGY = KID_BIT - 1;

/* Energy field mask for a width of bits (11, 16 or 30). */
__host__ __device__ __forceinline__ uint32_t energy_mask_of(uint32_t bits)
{
	return bits >= 30 ? 0x3fffffffu : (1u << bits) - 1;
}

enum : uint32_t {
	STREAM_INIT_CELL = 0,
	STREAM_INIT_AGENT = 1,
	STREAM_MOVE = 2,
	STREAM_ACT = 3,
};

/* Error bits raised on the device and read by the host after a step. */
enum : uint32_t {
	ERRF_OVERFLOW = 1u, /* agent pool too small for survivors + newborns */
	ERRF_TIMEOUT = 2u,  /* a look-back wait hit its iteration limit      */
};

/* Fused pipeline records (group buffers): key = destination cell within
 * its tile (bits 0-12) | move direction (bits 13-15; DIR_PARKED: not moved
 * because the run ended, DIR_DEAD: died in the move) | rank of the agent in
 * its source cell's list (bits 16-31); value = type | energy after the
 * move (before it for parked and dead records). */
constexpr uint32_t REC_DIR_SHIFT = 13;
constexpr uint32_t REC_RANK_SHIFT = 16;
constexpr uint32_t REC_RANK_MAX = 0xffffu;
constexpr uint32_t DIR_PARKED = 6;
constexpr uint32_t DIR_DEAD = 7;
/* Inbox entries per tile and parity: {group start, count | GROUP_GRAVE}. */
constexpr uint32_t IBX = 32;
constexpr uint32_t GROUP_GRAVE = 0x80000000u;

/* Philox4x32-10 (Salmon et al., SC'11), written from the paper. */
struct u4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ u4 philox4x32_10(u4 c, uint32_t k0,
	uint32_t k1)
{
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
	for (int r = 0; r < 10; r++) {
#ifdef __CUDA_ARCH__
		uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
		uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
#else
		uint64_t p0 = (uint64_t) 0xD2511F53u * c.x;
		uint64_t p1 = (uint64_t) 0xCD9E8D57u * c.z;
		uint32_t hi0 = (uint32_t) (p0 >> 32), lo0 = (uint32_t) p0;
		uint32_t hi1 = (uint32_t) (p1 >> 32), lo1 = (uint32_t) p1;
#endif
		u4 n;
		n.x = hi1 ^ c.y ^ k0;
		n.y = lo1;
		n.z = hi0 ^ c.w ^ k1;
		n.w = lo0;
		c = n;
		k0 += 0x9E3779B9u;
		k1 += 0xBB67AE85u;
	}
	return c;
}

/* Uniform integer in [0, n): floor(w * n / 2^32). */
__host__ __device__ __forceinline__ uint32_t draw(uint32_t w, uint32_t n)
{
#ifdef __CUDA_ARCH__
	return __umulhi(w, n);
#else
	return (uint32_t) (((uint64_t) w * n) >> 32);
#endif
}

/* The draw of (cell or agent number `id`, iteration, stream, rank k in the
 * cell's list) under the run's seed. */
__host__ __device__ __forceinline__ u4 rng(uint32_t seed_lo, uint32_t seed_hi,
	uint32_t id, uint32_t iter, uint32_t stream, uint32_t k)
{
	return philox4x32_10(u4{id, iter, stream, k}, seed_lo, seed_hi);
}

/* Unsigned division by a runtime constant d >= 1 via a precomputed
 * multiplier (Granlund & Montgomery, "Division by invariant integers
 * using multiplication", PLDI'94, round-up variant): q = umulhi(n, m) + n
 * >> s with m, s from fastdiv_make. Exact for all 32-bit n. */
struct fastdiv {
	uint32_t d, m, s;
};

inline fastdiv fastdiv_make(uint32_t d)
{
	fastdiv f;
	f.d = d;
	uint32_t l = 0;
	while (l < 32 && (1ull << l) < d) l++;
	/* m = floor(2^32 * (2^l - d) / d) + 1 */
	f.m = (uint32_t) (((1ull << 32) * ((1ull << l) - d)) / d + 1);
	f.s = l;
	return f;
}

__host__ __device__ __forceinline__ uint32_t fastdiv_div(uint32_t n, fastdiv f)
{
#ifdef __CUDA_ARCH__
	uint32_t t = __umulhi(n, f.m);
#else
	uint32_t t = (uint32_t) (((uint64_t) n * f.m) >> 32);
#endif
	/* (t + ((n - t) >> 1)) >> (s - 1) for s >= 1; s == 0 means d == 1. */
	if (f.s == 0) return n;
	return (t + ((n - t) >> 1)) >> (f.s - 1);
}

/* One simulation run inside a world (a world is one or many runs sharing
 * the agent arrays, the grass array and every launch). */
struct RunDev {
	uint32_t gx, gy, ncells;   /* grid                                     */
	uint32_t cbase;            /* first global cell, multiple of tile size */
	uint32_t first_tile, n_tiles;
	uint32_t sheep_gain, sheep_thr, sheep_prob;
	uint32_t wolves_gain, wolves_thr, wolves_prob;
	uint32_t restart;
	uint32_t seed_lo, seed_hi;
	uint32_t iters;            /* iterations this run performs             */
	uint32_t start_giter;      /* world iteration at which iter 1 runs - 1 */
	uint32_t active;           /* 0 = finished or empty slot               */
	uint32_t fbase;            /* this run's regrowth histogram (restart+1 slots) */
	uint32_t ss_from;          /* focal measures: steady state is t > ss_from */
	uint32_t emask;            /* energy field mask (2^width - 1)          */
	fastdiv gxdiv;
};

/* Running PPHPC focal measures of one run over its six outputs (sheep,
 * wolves, live grass, mean sheep energy, mean wolf energy, mean grass
 * countdown): max and min with the first iteration reaching them, and the
 * steady-state sum and sum of squares. */
struct FocalDev {
	double mx[6], mn[6], sum[6], sq[6];
	uint32_t amx[6], amn[6];
	uint32_t n, pad;
};

__host__ __device__ __forceinline__ void focal_outputs(uint32_t sheep,
	uint32_t wolves, uint32_t grass, uint64_t sheep_en, uint64_t wolves_en,
	uint64_t grass_en, uint32_t ncells, double o[6])
{
	o[0] = sheep;
	o[1] = wolves;
	o[2] = grass;
	o[3] = sheep ? (double) sheep_en / (double) sheep : 0.0;
	o[4] = wolves ? (double) wolves_en / (double) wolves : 0.0;
	o[5] = (double) grass_en / (double) ncells;
}

/* Fold the outputs of iteration t into f (t == first: start afresh). */
__host__ __device__ __forceinline__ void focal_fold(FocalDev &f, const double o[6],
	uint32_t t, bool first, uint32_t ss_from)
{
	if (first) {
		for (int k = 0; k < 6; k++) {
			f.mx[k] = f.mn[k] = o[k];
			f.amx[k] = f.amn[k] = t;
			f.sum[k] = f.sq[k] = 0.0;
		}
		f.n = 0;
	} else {
		for (int k = 0; k < 6; k++) {
			if (o[k] > f.mx[k]) { f.mx[k] = o[k]; f.amx[k] = t; }
			if (o[k] < f.mn[k]) { f.mn[k] = o[k]; f.amn[k] = t; }
		}
	}
	if (t > ss_from) {
		for (int k = 0; k < 6; k++) {
			f.sum[k] += o[k];
			f.sq[k] += o[k] * o[k];
		}
		f.n++;
	}
}

/* Per-world counters in device memory. The finish kernel's last CTA
 * advances the iteration and resets the per-launch counters for the next
 * one, so a whole iteration is a fixed launch sequence (captured as a
 * graph). */
struct WorldCounters {
	uint32_t n_agents;       /* agents after the last act (stats count)  */
	uint32_t giter;          /* world iterations completed               */
	uint32_t seq;            /* look-back epoch base, +1 per iteration   */
	uint32_t err;            /* ERRF_* bits                              */
	uint32_t xtop;           /* fused act: scratch slots taken by crowded tiles */
	uint32_t finish_done;    /* finish CTAs done                          */
	uint32_t sort_ticket[8]; /* one per radix pass                        */
	uint32_t aux_n;          /* element count of a standalone sort        */
	uint32_t fin_ticket;     /* finish chunk tickets                      */
	uint32_t n_all;          /* fused finish: records counted so far       */
	uint32_t tile_hi;        /* tiles [0, tile_hi) hold runs (fused act)   */
};

/* ---- memory-ordering helpers ---- */
__device__ __forceinline__ uint64_t ld_acquire_u64(const uint64_t *p)
{
	uint64_t v;
	asm volatile("ld.acquire.gpu.global.u64 %0, [%1];"
		: "=l"(v) : "l"(p) : "memory");
	return v;
}

__device__ __forceinline__ void st_release_u64(uint64_t *p, uint64_t v)
{
	asm volatile("st.release.gpu.global.u64 [%0], %1;"
		:: "l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint32_t ld_volatile_u32(const uint32_t *p)
{
	uint32_t v;
	asm volatile("ld.volatile.global.u32 %0, [%1];"
		: "=r"(v) : "l"(p) : "memory");
	return v;
}

/* Look-back words: [epoch:30 | flag:2 | value:32]. A word whose epoch is
 * not the current launch's epoch reads as "not yet published", so the
 * state arrays never need clearing between launches. */
constexpr uint64_t LB_FLAG_AGG = 1ull;
constexpr uint64_t LB_FLAG_PREFIX = 2ull;

__device__ __forceinline__ uint64_t lb_pack(uint32_t epoch, uint64_t flag,
	uint32_t value)
{
	return ((uint64_t) (epoch & 0x3fffffffu) << 34) | (flag << 32) | value;
}

/* Spin limit for every device-side wait: a wait that exceeds it raises
 * ERRF_TIMEOUT and proceeds (results are then invalid, the host reports
 * PP_ERR_TIMEOUT); no wait can hang the GPU. */
constexpr uint32_t SPIN_LIMIT = 1u << 22;

} /* namespace pp */
