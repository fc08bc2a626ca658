/*
 * pp_block.cuh -- block-level scan and decoupled look-back helpers shared
 * by the radix and act kernels (256-thread blocks).
 */
#pragma once

#include "pp_device.cuh"

namespace pp {

constexpr int BLOCK_THREADS = 256;

/* Exclusive block scan of one value per thread (256 threads). Returns the
 * exclusive prefix and writes the block total to *total. */
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v,
	uint32_t *total)
{
	__shared__ uint32_t ws[BLOCK_THREADS / 32];
	const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	uint32_t x = v;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
		if (lane >= (uint32_t) o) x += y;
	}
	if (lane == 31) ws[wid] = x;
	__syncthreads();
	if (wid == 0) {
		uint32_t s = lane < BLOCK_THREADS / 32 ? ws[lane] : 0;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
			if (lane >= (uint32_t) o) s += y;
		}
		if (lane < BLOCK_THREADS / 32) ws[lane] = s;
	}
	__syncthreads();
	uint32_t warp_prefix = wid ? ws[wid - 1] : 0;
	*total = ws[BLOCK_THREADS / 32 - 1];
	__syncthreads();
	return warp_prefix + x - v;
}

/* Decoupled look-back (Merrill & Garland, "Single-pass Parallel Prefix
 * Scan with Decoupled Look-back", 2016) for one counter of tile `tile`;
 * the counter of tile k lives at lb[k * stride]. Publishes the tile's
 * aggregate, walks back over predecessors until an inclusive prefix is
 * found, publishes its own inclusive prefix and returns the exclusive
 * one. Every wait is bounded by SPIN_LIMIT polls; on expiry ERRF_TIMEOUT
 * is raised in *err and the walk stops (the result is then invalid). */
__device__ __forceinline__ uint32_t lookback(uint64_t *lb, size_t stride,
	uint32_t tile, uint32_t agg, uint32_t epoch, uint32_t *err)
{
	if (tile == 0) {
		st_release_u64(&lb[0], lb_pack(epoch, LB_FLAG_PREFIX, agg));
		return 0;
	}
	st_release_u64(&lb[(size_t) tile * stride],
		lb_pack(epoch, LB_FLAG_AGG, agg));
	uint32_t acc = 0;
	int64_t k = (int64_t) tile - 1;
	uint32_t spins = 0;
	const uint32_t ep = epoch & 0x3fffffffu;
	while (k >= 0) {
		uint64_t word = ld_acquire_u64(&lb[(size_t) k * stride]);
		uint32_t wep = (uint32_t) (word >> 34);
		uint32_t flag = (uint32_t) (word >> 32) & 3u;
		if (wep != ep || flag == 0) {
			if (++spins > SPIN_LIMIT) {
				atomicOr(err, ERRF_TIMEOUT);
				break;
			}
			if (spins > 32) __nanosleep(64);
			continue;
		}
		acc += (uint32_t) word;
		if (flag == LB_FLAG_PREFIX) break;
		k--;
	}
	st_release_u64(&lb[(size_t) tile * stride],
		lb_pack(epoch, LB_FLAG_PREFIX, acc + agg));
	return acc;
}

/* The same look-back with four predecessor words in flight per step: the
 * walk over predecessors that have published only their aggregate costs a
 * quarter of the round trips. */
__device__ __forceinline__ uint32_t lookback4(uint64_t *lb, size_t stride,
	uint32_t tile, uint32_t agg, uint32_t epoch, uint32_t *err)
{
	if (tile == 0) {
		st_release_u64(&lb[0], lb_pack(epoch, LB_FLAG_PREFIX, agg));
		return 0;
	}
	st_release_u64(&lb[(size_t) tile * stride],
		lb_pack(epoch, LB_FLAG_AGG, agg));
	const uint32_t ep = epoch & 0x3fffffffu;
	uint32_t acc = 0;
	int64_t k = (int64_t) tile - 1;
	uint32_t spins = 0;
	while (k >= 0) {
		uint64_t wv[4];
#pragma unroll
		for (int q = 0; q < 4; q++)
			wv[q] = (k - q >= 0) ? ld_acquire_u64(&lb[(size_t) (k - q) * stride]) : 0;
		bool done = false;
		int used = 0;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			if (done || used != q) break;
			if (k - q < 0) { done = true; break; }
			uint32_t wep = (uint32_t) (wv[q] >> 34);
			uint32_t flag = (uint32_t) (wv[q] >> 32) & 3u;
			if (wep != ep || flag == 0) break;   /* not yet published */
			acc += (uint32_t) wv[q];
			used++;
			if (flag == LB_FLAG_PREFIX) done = true;
		}
		if (done) break;
		k -= used;
		if (used == 0) {
			if (++spins > SPIN_LIMIT) {
				atomicOr(err, ERRF_TIMEOUT);
				break;
			}
			if (spins > 32) __nanosleep(64);
		}
	}
	st_release_u64(&lb[(size_t) tile * stride],
		lb_pack(epoch, LB_FLAG_PREFIX, acc + agg));
	return acc;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

/* Full-warp sums with the warp reduction instruction (redux.sync). */
__device__ __forceinline__ uint32_t warp_sum(uint32_t v)
{
	return __reduce_add_sync(0xffffffffu, v);
}

/* 64-bit: three 22-bit chunks, whose 32-lane sums cannot overflow 32 bits;
 * the result is the sum modulo 2^64. */
__device__ __forceinline__ uint64_t warp_sum(uint64_t v)
{
	const uint32_t s0 = __reduce_add_sync(0xffffffffu, (uint32_t) v & 0x3fffffu);
	const uint32_t s1 = __reduce_add_sync(0xffffffffu, (uint32_t) (v >> 22) & 0x3fffffu);
	const uint32_t s2 = __reduce_add_sync(0xffffffffu, (uint32_t) (v >> 44));
	return (uint64_t) s0 + ((uint64_t) s1 << 22) + ((uint64_t) s2 << 44);
}

} /* namespace pp */
