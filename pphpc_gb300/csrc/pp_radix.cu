/*
 * pp_radix.cu -- stable LSD radix sort of (cell key, agent value) pairs.
 *
 * Replaces the cl_ops sort call of the reference (opencl/pp/pp_gpu.c:826-828,
 * bitonic by default, key `x >> 17` per pp_gpu.c:1798) with a one-sweep
 * style LSD radix sort:
 *   - the digit histograms of every pass come from one counting sweep
 *     (fused into the move kernel in the simulation; k_radix_hist here for
 *     standalone use);
 *   - each pass is one kernel: tiles of 4096 pairs are ranked per digit
 *     with warp ballots (one ballot per digit bit gives the set of lanes
 *     holding the same digit), warp-private digit counters in shared
 *     memory keep the ranks stable, tile digit offsets come from a
 *     decoupled look-back across tiles, and the tile is staged in shared
 *     memory in digit order so the global writes of each digit run are
 *     contiguous.
 * Keys are cell indices (or the dead sentinel), so only
 * ceil(log2(cells + 1)) bits are sorted.
 */
#include "pp_kernels.cuh"
#include "pp_block.cuh"

namespace pp {

__global__ void __launch_bounds__(256) k_radix_hist(const uint32_t *keys,
	const uint32_t *n_dev, uint32_t *hist, uint32_t d, uint32_t P)
{
	extern __shared__ uint32_t sh[];
	const uint32_t mask = (1u << d) - 1;
	for (uint32_t q = threadIdx.x; q < (P << d); q += blockDim.x) sh[q] = 0;
	__syncthreads();
	const uint32_t n = *n_dev;
	const uint32_t lane = threadIdx.x & 31;
	for (uint32_t base = blockIdx.x * blockDim.x; base < n;
		base += gridDim.x * blockDim.x) {
		uint32_t i = base + threadIdx.x;
		bool valid = i < n;
		uint32_t k = valid ? keys[i] : 0;
		/* one atomic per warp where the warp's digits agree (the high
		 * digits of nearly sorted keys), else one per lane (random keys:
		 * few collisions) */
		const uint32_t vmask = __ballot_sync(0xffffffffu, valid);
		for (uint32_t p = 0; p < P; p++) {
			const uint32_t dig = (k >> (p * d)) & mask;
			const uint32_t d0 = __shfl_sync(0xffffffffu, dig, 0);
			if (__all_sync(0xffffffffu, !valid || dig == d0)) {
				if (lane == 0 && vmask) atomicAdd(&sh[(p << d) + d0], __popc(vmask));
			} else if (valid) {
				atomicAdd(&sh[(p << d) + dig], 1u);
			}
		}
	}
	__syncthreads();
	for (uint32_t q = threadIdx.x; q < (P << d); q += blockDim.x) {
		uint32_t c = sh[q];
		if (c) atomicAdd(&hist[(q >> d) * 256 + (q & mask)], c);
	}
}

__device__ __forceinline__ uint32_t lanemask_lt()
{
	uint32_t m;
	asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
	return m;
}

template <int DBITS>
__global__ void __launch_bounds__(SORT_THREADS, 3) k_radix_pass(
	const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
	uint32_t *__restrict__ kout, uint32_t *__restrict__ vout,
	const uint32_t *__restrict__ hist_pass, uint64_t *lb, WorldCounters *ctr,
	const uint32_t *n_dev, uint32_t pass, uint32_t shift)
{
	constexpr uint32_t RADIX = 1u << DBITS;
	constexpr uint32_t WARPS = SORT_THREADS / 32;
	constexpr uint32_t MASK = RADIX - 1;
	__shared__ uint32_t s_digit_base[RADIX];
	__shared__ uint32_t s_wcnt[WARPS][RADIX];
	__shared__ uint32_t s_tile_start[RADIX];
	__shared__ uint32_t s_gpos[RADIX];
	__shared__ uint32_t s_stage_k[SORT_TILE];
	__shared__ uint32_t s_stage_v[SORT_TILE];
	__shared__ uint32_t s_tile;

	const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const uint32_t n = *n_dev;
	const uint32_t num_tiles = (n + SORT_TILE - 1) / SORT_TILE;
	const uint32_t epoch = ctr->seq * 8u + pass;

	/* Global start of every digit: exclusive scan of this pass's counts. */
	{
		uint32_t c = tid < RADIX ? hist_pass[tid] : 0;
		uint32_t tot;
		uint32_t ex = block_excl_scan(c, &tot);
		if (tid < RADIX) s_digit_base[tid] = ex;
	}

	const uint32_t lt = lanemask_lt();
	for (;;) {
		if (tid == 0) s_tile = atomicAdd(&ctr->sort_ticket[pass], 1u);
		for (uint32_t q = tid; q < WARPS * RADIX; q += SORT_THREADS)
			(&s_wcnt[0][0])[q] = 0;
		__syncthreads();
		const uint32_t tile = s_tile;
		if (tile >= num_tiles) break;

		uint32_t k[SORT_IPT], v[SORT_IPT], rk[SORT_IPT];
		const uint32_t wbase = tile * SORT_TILE + warp * 32 * SORT_IPT;
#pragma unroll
		for (int j = 0; j < SORT_IPT; j++) {
			uint32_t idx = wbase + j * 32 + lane;
			bool valid = idx < n;
			k[j] = valid ? kin[idx] : 0xffffffffu;
			v[j] = valid ? vin[idx] : 0;
		}
		/* Stable warp-level ranking, items in (j, lane) order. */
#pragma unroll
		for (int j = 0; j < SORT_IPT; j++) {
			uint32_t idx = wbase + j * 32 + lane;
			bool valid = idx < n;
			uint32_t dg = (k[j] >> shift) & MASK;
			uint32_t peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
			for (int b = 0; b < DBITS; b++) {
				uint32_t bit = (dg >> b) & 1u;
				uint32_t bb = __ballot_sync(0xffffffffu, bit);
				peers &= bit ? bb : ~bb;
			}
			uint32_t below = __popc(peers & lt);
			uint32_t base = valid ? s_wcnt[warp][dg] : 0;
			__syncwarp();
			if (valid && below == 0) s_wcnt[warp][dg] = base + __popc(peers);
			__syncwarp();
			rk[j] = base + below;
		}
		__syncthreads();
		/* Per digit: exclusive offsets across warps and the tile count. */
		uint32_t cnt = 0;
		if (tid < RADIX) {
#pragma unroll
			for (uint32_t w = 0; w < WARPS; w++) {
				uint32_t c = s_wcnt[w][tid];
				s_wcnt[w][tid] = cnt;
				cnt += c;
			}
		}
		uint32_t tot;
		uint32_t tstart = block_excl_scan(cnt, &tot);
		if (tid < RADIX) {
			s_tile_start[tid] = tstart;
			uint32_t ex = lookback4(lb + tid, RADIX, tile, cnt, epoch,
				&ctr->err);
			s_gpos[tid] = s_digit_base[tid] + ex;
		}
		__syncthreads();
		/* Stage the tile in digit order. */
#pragma unroll
		for (int j = 0; j < SORT_IPT; j++) {
			uint32_t idx = wbase + j * 32 + lane;
			if (idx < n) {
				uint32_t dg = (k[j] >> shift) & MASK;
				uint32_t pos = s_tile_start[dg] + s_wcnt[warp][dg] + rk[j];
				s_stage_k[pos] = k[j];
				s_stage_v[pos] = v[j];
			}
		}
		__syncthreads();
		const uint32_t tile_n = min((uint32_t) SORT_TILE, n - tile * SORT_TILE);
		for (uint32_t q = tid; q < tile_n; q += SORT_THREADS) {
			uint32_t kk = s_stage_k[q];
			uint32_t dg = (kk >> shift) & MASK;
			uint32_t gp = s_gpos[dg] + q - s_tile_start[dg];
			kout[gp] = kk;
			vout[gp] = s_stage_v[q];
		}
		__syncthreads();
	}
}

cudaError_t launch_radix_hist(const uint32_t *keys, const uint32_t *n_dev,
	uint32_t *hist, uint32_t digit_bits, uint32_t passes, int blocks,
	cudaStream_t s)
{
	size_t smem = (size_t) (passes << digit_bits) * sizeof(uint32_t);
	k_radix_hist<<<blocks, 256, smem, s>>>(keys, n_dev, hist, digit_bits,
		passes);
	return cudaGetLastError();
}

cudaError_t launch_radix_pass(const uint32_t *kin, const uint32_t *vin,
	uint32_t *kout, uint32_t *vout, const uint32_t *hist_pass,
	uint64_t *lb, WorldCounters *ctr, const uint32_t *n_dev, uint32_t pass,
	uint32_t shift, uint32_t digit_bits, int blocks, cudaStream_t s)
{
	switch (digit_bits) {
	case 5: k_radix_pass<5><<<blocks, SORT_THREADS, 0, s>>>(kin, vin, kout, vout, hist_pass, lb, ctr, n_dev, pass, shift); break;
	case 6: k_radix_pass<6><<<blocks, SORT_THREADS, 0, s>>>(kin, vin, kout, vout, hist_pass, lb, ctr, n_dev, pass, shift); break;
	case 7: k_radix_pass<7><<<blocks, SORT_THREADS, 0, s>>>(kin, vin, kout, vout, hist_pass, lb, ctr, n_dev, pass, shift); break;
	case 8: k_radix_pass<8><<<blocks, SORT_THREADS, 0, s>>>(kin, vin, kout, vout, hist_pass, lb, ctr, n_dev, pass, shift); break;
	default: return cudaErrorInvalidValue;
	}
	return cudaGetLastError();
}

} /* namespace pp */

namespace pp {

int occupancy_sort(int dbits)
{
	int n = 0;
	cudaError_t e;
	switch (dbits) {
	case 5: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_radix_pass<5>, SORT_THREADS, 0); break;
	case 6: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_radix_pass<6>, SORT_THREADS, 0); break;
	case 7: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_radix_pass<7>, SORT_THREADS, 0); break;
	default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_radix_pass<8>, SORT_THREADS, 0); break;
	}
	if (e != cudaSuccess) { cudaGetLastError(); return 1; }
	return n;
}

} /* namespace pp */
