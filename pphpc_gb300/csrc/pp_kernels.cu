/*
 * pp_kernels.cu -- the per-iteration simulation kernels for sm_103a.
 *
 *   k_regions     move_agent (opencl/pp/pp_gpu.cl:744-821): the agents of
 *                 each tile's region, moved into the dense sort input, plus
 *                 the digit histograms of every radix pass (replaces the
 *                 upfront histogram pass of the sort).
 *   k_offsets     find_cell_idx (pp_gpu.cl:834-867): start index of every
 *                 bucket (a tile of cells, or a single cell) in the
 *                 cell-sorted agent array.
 *   k_act         grass (pp_gpu.cl:448-476) + action_agent
 *                 (pp_gpu.cl:883-979), fused per tile of cells: countdown,
 *                 in-cell conflict resolution in priority order, newborn
 *                 slots by a block prefix sum, survivors and newborns
 *                 written to the tile's own region (no inter-tile wait),
 *                 per-tile partial stats.
 *   k_finish      reduce_grass1/2 + reduce_agent1/2 (pp_gpu.cl:485-736):
 *                 per-tile partial stats summed per run into the stats
 *                 ring; scan of the region counts into dense bases
 *                 (decoupled look-back across chunks of tiles); its last
 *                 CTA advances the iteration.
 *   k_init_*      init_cell / init_agent (pp_gpu.cl:368-439).
 *
 * Draws are keyed by (cell, rank of the agent in its cell's list), never by
 * an array position. Every kernel reads its sizes from device memory, so an
 * iteration is a fixed launch sequence, captured once as a CUDA graph.
 */
#include <algorithm>
#include <type_traits>

#include "pp_kernels.cuh"
#include "pp_block.cuh"
#include "pp_act.cuh"

namespace pp {

/* ------------------------------------------------------------------ */
/* Move                                                                */
/* ------------------------------------------------------------------ */

/* One warp per tile region: the tile's agents (cell-sorted lists) from the
 * region buffer. MOVE: the move of every agent (draw keyed by cell and
 * rank in the cell's list; ranks from a ballot of list starts with a carry
 * across 32-agent chunks) into the dense sort input B at the tile's dense
 * base, plus the digit histograms of every radix pass. !MOVE: a plain copy
 * into the dense array ko/vo (state read-back). */
template <bool MOVE>
__global__ void __launch_bounds__(256) k_regions(WorldDev w, uint32_t *ko,
	uint32_t *vo)
{
	extern __shared__ uint32_t sh_hist[];
	const uint32_t d = w.digit_bits, P = w.passes, mask = (1u << d) - 1;
	if (MOVE) {
		for (uint32_t q = threadIdx.x; q < (P << d); q += blockDim.x)
			sh_hist[q] = 0;
		__syncthreads();
	}
	const uint32_t g = w.ctr->giter + 1;
	const uint32_t lane = threadIdx.x & 31;
	const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
	for (uint32_t tile = gw; tile < w.n_tiles; tile += nw) {
		const uint32_t cnt = w.rcnt[tile];
		if (cnt == 0) continue;
		const uint32_t rs = w.rstart[tile], db = w.dbase[tile];
		const RunDev &run = w.runs[w.tile_run[tile]];
		const uint32_t t = g - run.start_giter;
		const bool live = run_live(run, t);
		uint32_t carry_key = 0xffffffffu, carry_rank = 0;
		for (uint32_t j0 = 0; j0 < cnt; j0 += 32) {
			const uint32_t j = j0 + lane;
			const bool valid = j < cnt;
			/* past an overflow of the pool (its error is already raised)
			 * the dense positions run beyond it: nothing is written there
			 * and nothing counted */
			const bool keep = valid && db + j < w.cap;
			const uint32_t key = valid ? w.kR[rs + j] : 0xffffffffu;
			const uint32_t val = valid ? w.vR[rs + j] : 0;
			uint32_t prev = __shfl_up_sync(0xffffffffu, key, 1);
			if (lane == 0) prev = carry_key;
			const uint32_t starts = __ballot_sync(0xffffffffu, valid && key != prev);
			const uint32_t upto = starts & (0xffffffffu >> (31 - lane));
			const uint32_t k = upto ? lane - (31 - __clz(upto)) : carry_rank + 1 + lane;
			const uint32_t last = min(31u, cnt - j0 - 1);
			carry_key = __shfl_sync(0xffffffffu, key, last);
			carry_rank = __shfl_sync(0xffffffffu, k, last);
			if (!MOVE) {
				if (keep) {
					ko[db + j] = key;
					vo[db + j] = val;
				}
				continue;
			}
			uint32_t nk = 0xffffffffu, nv = 0;
			if (keep) {
				if (live) move_one(run, key, val, k, t, w.dead_key, nk, nv);
				else { nk = w.dead_key; nv = val & TYPE_BIT; }
				w.kB[db + j] = nk;
				w.vB[db + j] = nv;
			}
			/* Digit counts: one atomic per warp when the warp's digits
			 * agree (the high digits of a nearly cell-sorted array), else
			 * one per lane. */
			const uint32_t vmask = __ballot_sync(0xffffffffu, keep);
			for (uint32_t p = 0; p < P; p++) {
				uint32_t dig = (nk >> (w.sort_shift + p * d)) & mask;
				uint32_t d0 = __shfl_sync(0xffffffffu, dig, 0);
				bool same = __all_sync(0xffffffffu, !keep || dig == d0);
				if (same) {
					if (lane == 0) atomicAdd(&sh_hist[(p << d) + d0], __popc(vmask));
				} else if (keep) {
					atomicAdd(&sh_hist[(p << d) + dig], 1u);
				}
			}
		}
	}
	if (MOVE) {
		__syncthreads();
		for (uint32_t q = threadIdx.x; q < (P << d); q += blockDim.x) {
			uint32_t c = sh_hist[q];
			if (c) atomicAdd(&w.hist[(q >> d) * 256 + (q & mask)], c);
		}
	}
}

/* Move of one run alone (kernel-level check) over a cell-sorted array. */
__global__ void k_move_only(const uint32_t *kin, const uint32_t *vin,
	uint32_t *kout, uint32_t *vout, uint32_t n, const RunDev *run_dev,
	uint32_t t, uint32_t dead_key)
{
	const RunDev run = *run_dev;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
		i += gridDim.x * blockDim.x) {
		uint32_t k = 0;
		while (k < i && kin[i - k - 1] == kin[i]) k++;
		uint32_t nk, nv;
		move_one(run, kin[i], vin[i], k, t, dead_key, nk, nv);
		kout[i] = nk;
		vout[i] = nv;
	}
}

/* ------------------------------------------------------------------ */
/* Bucket offsets                                                      */
/* ------------------------------------------------------------------ */

/* off[b] = first index whose key >> log_tile >= b, for b = 0..n_buckets.
 * Keys are sorted; keys >> log_tile above n_buckets clamp to n_buckets.
 * Each index writes the offsets of the buckets between its predecessor's
 * bucket and its own, so every entry is written exactly once. */
__global__ void k_offsets(const uint32_t *keys, const uint32_t *n_dev,
	uint32_t log_tile, uint32_t n_buckets, uint32_t *off)
{
	const uint32_t n = *n_dev;
	const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
	if (n == 0) {
		for (uint32_t b = tid; b <= n_buckets; b += gridDim.x * blockDim.x)
			off[b] = 0;
		return;
	}
	for (uint32_t i = tid; i < n; i += gridDim.x * blockDim.x) {
		uint32_t b = min(keys[i] >> log_tile, n_buckets);
		uint32_t lo = (i == 0) ? 0 : min(keys[i - 1] >> log_tile, n_buckets) + 1;
		for (uint32_t q = lo; q <= b; q++) off[q] = i;
		if (i == n - 1)
			for (uint32_t q = b + 1; q <= n_buckets; q++) off[q] = n;
	}
}

/* ------------------------------------------------------------------ */
/* Act                                                                 */
/* ------------------------------------------------------------------ */

/* First index in a[0, m) with a[i] >= x. */
__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t *a,
	uint32_t m, uint32_t x)
{
	uint32_t lo = 0, hi = m;
	while (lo < hi) {
		uint32_t mid = (lo + hi) >> 1;
		if (a[mid] < x) lo = mid + 1;
		else hi = mid;
	}
	return lo;
}

/* Warp-wide decoupled look-back (lanes read 32 predecessors at once).
 * Called by all lanes of one warp; returns the exclusive prefix of `tile`
 * and publishes its inclusive prefix. Bounded: a predecessor that does not
 * publish within `limit` polls raises ERRF_TIMEOUT. */
__device__ uint32_t warp_lookback(uint64_t *lb, uint32_t tile, uint32_t agg,
	uint32_t epoch, uint32_t *err, uint32_t limit = SPIN_LIMIT)
{
	const uint32_t lane = threadIdx.x & 31;
	if (tile == 0) {
		if (lane == 0) st_release_u64(&lb[0], lb_pack(epoch, LB_FLAG_PREFIX, agg));
		return 0;
	}
	if (lane == 0) st_release_u64(&lb[tile], lb_pack(epoch, LB_FLAG_AGG, agg));
	const uint32_t ep = epoch & 0x3fffffffu;
	uint32_t acc = 0;
	int64_t end = (int64_t) tile;     /* window covers end-32 .. end-1 */
	uint32_t spins = 0;
	bool timed_out = false;
	while (end > 0) {
		int64_t idx = end - 1 - (int64_t) lane;
		uint32_t flag, val;
		for (;;) {
			if (idx >= 0) {
				uint64_t word = ld_acquire_u64(&lb[idx]);
				bool cur = (uint32_t) (word >> 34) == ep;
				flag = cur ? ((uint32_t) (word >> 32) & 3u) : 0u;
				val = (uint32_t) word;
			} else {
				flag = (uint32_t) LB_FLAG_PREFIX;  /* before tile 0 */
				val = 0;
			}
			if (__all_sync(0xffffffffu, flag != 0)) break;
			if (++spins > limit) { timed_out = true; break; }
			if (spins > 32) __nanosleep(64);
		}
		if (timed_out) {
			if (lane == 0) atomicOr(err, ERRF_TIMEOUT);
			break;
		}
		uint32_t pm = __ballot_sync(0xffffffffu, flag == LB_FLAG_PREFIX);
		if (pm) {
			uint32_t first = __ffs(pm) - 1;      /* nearest inclusive prefix */
			uint32_t v = lane <= first ? val : 0;
			acc += warp_sum(v);
			break;
		}
		acc += warp_sum(val);
		end -= 32;
	}
	if (lane == 0)
		st_release_u64(&lb[tile], lb_pack(epoch, LB_FLAG_PREFIX, acc + agg));
	return acc;
}

/* One CTA per tile of CPT * 256 cells (tiles do not depend on each other).
 * Phases:
 *   (grouping)    the tile's agents arrive grouped by tile in canonical
 *                 order; a counting sort by cell in shared memory
 *                 (counters transposed across threads so no two threads of
 *                 a warp share a bank), each cell's short list put back in
 *                 arrival order;
 *   B (per agent) priority and dice of every agent (its rank = distance
 *                 to its cell's first entry);
 *   C (per occupied cell, from its first agent) the cell's grass
 *                 countdown (from its regrowth iteration) and actions;
 *   E (per agent chunk) survivors and newborns, in list order, into the
 *                 tile's region [2 * a0, 2 * a0 + total), agent stats.
 * Cells without agents are not touched: the countdown decrement of
 * pp_gpu.cl:448-476 is implicit in the regrowth representation. */
template <int CPT>
__global__ void __launch_bounds__(ACT_THREADS, 5) k_act(WorldDev w,
	const uint32_t *__restrict__ kS, uint32_t *__restrict__ vS)
{
	extern __shared__ uint32_t sm[];
	uint32_t *sk = sm, *sv = sm + w.act_cap, *sp = sv + w.act_cap,
		*sd = sp + w.act_cap, *sperm = sd + w.act_cap;
	uint32_t *scnt = sperm + w.act_cap;                 /* CPT * 256 */
	const uint32_t tid = threadIdx.x;
	const uint32_t tile = blockIdx.x;   /* tiles are independent */
	const uint32_t g = w.ctr->giter + 1;
	const RunDev &run = w.runs[w.tile_run[tile]];
	const uint32_t t = g - run.start_giter;
	/* a world whose agent pool has overflowed is failed (the host returns
	 * PP_OUT_OF_RESOURCES at its next check): its later acts do nothing */
	if (!run_live(run, t) || (w.ctr->err & ERRF_OVERFLOW)) {
		/* finished run, free tile space or a failed world: no agents
		 * survive, no stats */
		if (tid == 0) {
			w.rstart[tile] = 0;
			w.rcnt[tile] = 0;
		}
		if (tid < 8) w.part[(size_t) tile * 8 + tid] = 0;
		return;
	}
	const uint32_t seed_lo = run.seed_lo, seed_hi = run.seed_hi;
	const uint32_t cbase = run.cbase;
	ActParams ap;
	ap.sheep_gain = run.sheep_gain; ap.sheep_thr = run.sheep_thr;
	ap.sheep_prob = run.sheep_prob; ap.wolves_gain = run.wolves_gain;
	ap.wolves_thr = run.wolves_thr; ap.wolves_prob = run.wolves_prob;
	ap.restart = run.restart;
	ap.emask = run.emask;
	const uint32_t c0 = tile << w.log_tile;
	const uint32_t lt0 = c0 - cbase;          /* run-local index of the tile start */
	const uint32_t a0 = w.tile_off[tile], a1 = w.tile_off[tile + 1];
	const uint32_t m = a1 - a0;
	const bool in_smem = m <= w.act_cap;
	/* The sort grouped agents by tile only, in canonical order (source
	 * cell, source rank); group them by cell here, keeping that order.
	 * The phases are instantiated once for a tile whose arrays are in
	 * shared memory and once for a crowded tile's global arrays, so each
	 * copy addresses one memory space directly. */
	auto phases = [&](auto smem_tag, uint32_t *UK, uint32_t *UV, uint32_t *PERM,
		uint32_t *LK, uint32_t *LV, uint32_t *LP, uint32_t *LD) {
		constexpr bool SMEM = decltype(smem_tag)::value;
		if (SMEM) {
			for (uint32_t j = tid; j < m; j += ACT_THREADS) {
				UK[j] = kS[a0 + j];
				UV[j] = vS[a0 + j];
			}
		}
		/* per-cell counters, transposed like the countdowns: cell c lives at
		 * SLOT(c) = (c % CPT) * 256 + c / CPT, so no two threads of a warp
		 * share a bank */
#define SLOT(c) ((((c) % CPT) * ACT_THREADS) + (c) / CPT)
#pragma unroll
		for (int q = 0; q < CPT; q++) scnt[q * ACT_THREADS + tid] = 0;
		__syncthreads();
		/* counting sort of the tile's agents by cell */
		for (uint32_t j = tid; j < m; j += ACT_THREADS) {
			const uint32_t lc = UK[j] - c0;
			atomicAdd(&scnt[SLOT(lc)], 1u);
		}
		__syncthreads();
		{
			uint32_t loc = 0;
#pragma unroll
			for (int q = 0; q < CPT; q++) {
				loc += scnt[q * ACT_THREADS + tid];
			}
			uint32_t tot;
			uint32_t run_start = block_excl_scan(loc, &tot);
#pragma unroll
			for (int q = 0; q < CPT; q++) {
				uint32_t c = scnt[q * ACT_THREADS + tid];
				scnt[q * ACT_THREADS + tid] = run_start;
				run_start += c;
			}
		}
		__syncthreads();
		for (uint32_t j = tid; j < m; j += ACT_THREADS) {
			const uint32_t lc = UK[j] - c0;
			PERM[atomicAdd(&scnt[SLOT(lc)], 1u)] = j;
		}
		__syncthreads();
		/* scnt[SLOT(c)] is now the end of cell c, whose agents occupy [end of
		 * c - 1, end of c) in the order of the atomics; each goes to the cell's
		 * start plus its rank in arrival order, which only an agent sharing
		 * its cell has to count. LK holds the cell in bits 0-15 and the rank
		 * in the cell's list in bits 16-31. */
		for (uint32_t i = tid; i < m; i += ACT_THREADS) {
			const uint32_t j = PERM[i];
			const uint32_t lc = UK[j] - c0;
			const uint32_t e = scnt[SLOT(lc)], b = lc ? scnt[SLOT(lc - 1)] : 0;
			uint32_t d = i;
			if (e - b > 1) {
				d = b;
				for (uint32_t q = b; q < e; q++) d += PERM[q] < j;
			}
			if (d - b > 0xffffu) atomicOr(&w.ctr->err, ERRF_OVERFLOW);
			LK[d] = lc | (d - b) << 16;
			LV[d] = UV[j];
		}
#undef SLOT
		__syncthreads();
		/* B: draws of every agent, and its cell's countdown max(0, regrowth -
		 * t) read before any sheep eats (LD = dice | countdown << 7) */
		const uint16_t t16 = (uint16_t) t;
		for (uint32_t j = tid; j < m; j += ACT_THREADS) {
			const uint32_t lk = LK[j], lc = lk & 0xffffu;
			u4 r = rng(seed_lo, seed_hi, lt0 + lc, t, STREAM_ACT, lk >> 16);
			const int32_t dd = (int16_t) (uint16_t) (w.grass[c0 + lc] - t16);
			LP[j] = r.x;
			LD[j] = draw(r.y, 100) | (dd > 0 ? (uint32_t) dd << 7 : 0u);
		}
		__syncthreads();
		/* C: actions, one thread per agent; a sheep that eats sets its cell's
		 * regrowth to t + restart, counted for the run's regrowth histogram */
		uint32_t eats = 0;
		for (uint32_t j = tid; j < m; j += ACT_THREADS) {
			const uint32_t lk = LK[j], lc = lk & 0xffffu;
			const uint32_t p = j - (lk >> 16);
			uint32_t e = j + 1;
			while (e < m && (LK[e] >> 16) != 0) e++;
			const uint32_t dg = LD[j];
			uint32_t kid;
			if (act_agent(j, p, e, LV, LP, ap, dg >> 7, dg & 127u, &kid)) {
				w.grass[c0 + lc] = (uint16_t) (t16 + (uint16_t) ap.restart);
				eats++;
			}
			LD[j] = kid;
		}
		__syncthreads();
		/* E: outputs in list order, contiguous agent chunks per thread */
		const uint32_t ch = (m + ACT_THREADS - 1) / ACT_THREADS;
		const uint32_t ja = min(tid * ch, m), jb = min(ja + ch, m);
		uint32_t cnt = 0;
		for (uint32_t j = ja; j < jb; j++)
			cnt += ((LV[j] & EATEN_BIT) == 0) + ((LD[j] & KID_BIT) != 0);
		uint32_t total;
		const uint32_t excl = block_excl_scan(cnt, &total);
		const uint32_t rs = 2 * a0;
		if (tid == 0) {
			w.rstart[tile] = rs;
			w.rcnt[tile] = total;
		}
		uint32_t o = rs + excl;
		uint32_t sheep = 0, wolves = 0;
		uint64_t sen = 0, wen = 0;
		for (uint32_t j = ja; j < jb; j++) {
			const uint32_t v = LV[j], k = (LK[j] & 0xffffu) + c0, kd = LD[j];
			const uint32_t tb = v & TYPE_BIT, en = v & ENERGY_MASK;
			if (!(v & EATEN_BIT)) {
				w.kR[o] = k;
				w.vR[o] = v;
				o++;
				if (tb) { wolves++; wen += en; }
				else { sheep++; sen += en; }
			}
			if (kd & KID_BIT) {
				const uint32_t ke = kd & KID_ENERGY;
				w.kR[o] = k;
				w.vR[o] = tb | ke;
				o++;
				if (tb) { wolves++; wen += ke; }
				else { sheep++; sen += ke; }
			}
		}
		/* per-tile partial stats; the tile's eating events go to the run's
		 * regrowth histogram slot of iteration t + restart */
		{
			__shared__ uint64_t red[5][ACT_THREADS / 32];
			const uint32_t lane = tid & 31, wid = tid >> 5;
			const uint32_t sw = warp_sum(sheep | (wolves << 16));
			const uint32_t ew = warp_sum(eats);
			const uint64_t se = warp_sum(sen), we = warp_sum(wen);
			if (lane == 0) {
				red[0][wid] = sw & 0xffffu;
				red[1][wid] = sw >> 16;
				red[2][wid] = ew;
				red[3][wid] = se;
				red[4][wid] = we;
			}
			__syncthreads();
			if (tid < 5) {
				uint64_t sum = 0;
				for (uint32_t q = 0; q < ACT_THREADS / 32; q++) sum += red[tid][q];
				if (tid == 2) {
					if (sum)
						atomicAdd(&w.fring[run.fbase + (t + ap.restart) % (ap.restart + 1)],
							(uint32_t) sum);
					w.part[(size_t) tile * 8 + 2] = 0;
					w.part[(size_t) tile * 8 + 5] = 0;
				} else {
					w.part[(size_t) tile * 8 + tid] = sum;
				}
			}
		}
	};
	if (in_smem)
		phases(std::true_type{}, sk, sv, sperm, sp, sd, sk, sv);
	else
		phases(std::false_type{}, const_cast<uint32_t *>(kS) + a0, vS + a0,
			w.scratch_perm + a0, w.scratch_key + a0, w.scratch_val + a0,
			w.scratch_prio + a0, w.scratch_kid + a0);
}

/* Per chunk of tiles (chunks taken by ticket, so a chunk's predecessors are
 * always running or done):
 *   FULL: the chunk's per-tile partial stats summed per run into this
 *         iteration's stats ring row (reduce_grass/agent, pp_gpu.cl:485-736);
 *   the exclusive scan of the tiles' region counts into their dense bases
 *   (decoupled look-back across chunks); the total becomes n_agents, and a
 *   total above the agent pool raises ERRF_OVERFLOW (pp_gpu.c:847-852);
 *   the last CTA resets the per-launch counters (FULL: advances the
 *   iteration, clears the histograms and the next stats row). */
template <bool FULL, bool FUSED>
__global__ void __launch_bounds__(256) k_finish(WorldDev w)
{
	__shared__ uint32_t s_chunk, s_last, s_base;
	__shared__ uint64_t s_part[6];
	if (threadIdx.x == 0) s_chunk = atomicAdd(&w.ctr->fin_ticket, 1u);
	__syncthreads();
	const uint32_t chunk = s_chunk;
	const uint32_t g = w.ctr->giter + 1;
	const uint32_t row = g % w.ring_rows;
	const uint32_t epoch = w.ctr->seq * 8u + 7u;
	/* fused pipeline: only tiles below the high-water mark hold runs */
	const uint32_t nt = FUSED ? min(w.ctr->tile_hi, w.n_tiles) : w.n_tiles;
	const uint32_t per = (nt + gridDim.x - 1) / gridDim.x;
	const uint32_t t0 = min(chunk * per, nt);
	const uint32_t t1 = min(t0 + per, nt);
	if (FULL) {
		const uint32_t r0 = t0 < t1 ? w.tile_run[t0] : 0;
		bool same = true;
		for (uint32_t tl = t0 + threadIdx.x; tl < t1; tl += blockDim.x)
			same &= w.tile_run[tl] == r0;
		same = __syncthreads_and(same);
		if (same) {
			/* one run: block reduction, one atomic per field */
			uint64_t v[6] = {0, 0, 0, 0, 0, 0};
			for (uint32_t tl = t0 + threadIdx.x; tl < t1; tl += blockDim.x) {
#pragma unroll
				for (int f = 0; f < 6; f++) v[f] += w.part[(size_t) tl * 8 + f];
			}
			StatAcc a;
			a.sheep = (uint32_t) v[0]; a.wolves = (uint32_t) v[1];
			a.galive = (uint32_t) v[2]; a.sen = v[3]; a.wen = v[4]; a.gen = v[5];
			block_stats(a, s_part);
			if (threadIdx.x < 6 && t0 < t1)
				stats_atomic_add(&w.ring[(size_t) row * w.nruns_cap + r0],
					threadIdx.x, s_part[threadIdx.x]);
		} else {
			for (uint32_t tl = t0 + threadIdx.x; tl < t1; tl += blockDim.x) {
				PPStatistics *dst = &w.ring[(size_t) row * w.nruns_cap + w.tile_run[tl]];
				for (int f = 0; f < 6; f++)
					stats_atomic_add(dst, f, w.part[(size_t) tl * 8 + f]);
			}
		}
	}
	if (FULL) {
		/* grass stats of iteration t of every live run from its regrowth
		 * histogram: pending regrowths r in (t, t + restart] are the dead
		 * cells, each with countdown r - t. Slot t (cells alive again since
		 * t) is cleared for the eating events of iteration t + 1, which
		 * land at t + 1 + restart = t (mod restart + 1). */
		for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < w.nruns_cap;
			r += gridDim.x * blockDim.x) {
			const RunDev &run = w.runs[r];
			const uint32_t t = g - run.start_giter;
			if (!run_live(run, t)) continue;
			const uint32_t fs = run.restart + 1;
			uint32_t *f = w.fring + run.fbase;
			uint64_t dead = 0, sum = 0;
			for (uint32_t k = 1; k <= run.restart; k++) {
				const uint32_t c = f[(t + k) % fs];
				dead += c;
				sum += (uint64_t) k * c;
			}
			PPStatistics *dst = &w.ring[(size_t) row * w.nruns_cap + r];
			stats_atomic_add(dst, 2, run.ncells - dead);
			stats_atomic_add(dst, 5, sum);
			f[t % fs] = 0;
		}
	}
	/* dense bases: of the regions (sort pipeline), or of the next act's
	 * inputs, counted from the groups posted to each tile's inbox (fused
	 * pipeline; the next act writes its groups at twice its base) */
	const uint32_t pnext = FULL ? (g + 1) & 1 : g & 1;
	uint32_t all = 0;    /* fused: every posted record (dead ones too) */
	auto tile_count = [&](uint32_t tl) -> uint32_t {
		if (!FUSED) return w.rcnt[tl];
		const size_t ib = (size_t) pnext * w.n_tiles + tl;
		const uint32_t n = min(w.inbox_n[ib], IBX);
		uint32_t c = 0;
		for (uint32_t i = 0; i < n; i++) {
			const uint32_t y = w.inbox[ib * IBX + i].y;
			c += (y & GROUP_GRAVE) ? 0u : y;
			all += y & ~GROUP_GRAVE;
		}
		return c;
	};
	const uint32_t tpt = (per + blockDim.x - 1) / blockDim.x;
	const uint32_t ta = min(t0 + threadIdx.x * tpt, t1), tb = min(ta + tpt, t1);
	/* a thread's first tiles keep their counts in registers for the base
	 * writes below */
	constexpr uint32_t KEEP = 4;
	uint32_t kept[KEEP];
	uint32_t local = 0;
#pragma unroll
	for (uint32_t q = 0; q < KEEP; q++) {
		kept[q] = ta + q < tb ? tile_count(ta + q) : 0u;
		local += kept[q];
	}
	for (uint32_t tl = ta + KEEP; tl < tb; tl++) local += tile_count(tl);
	if (FUSED) {
		/* the agent count after the act: all records, summed per CTA */
		const uint32_t a = warp_sum(all);
		if ((threadIdx.x & 31) == 0 && a) atomicAdd(&w.ctr->n_all, a);
	}
	uint32_t total;
	const uint32_t excl = block_excl_scan(local, &total);
	if (threadIdx.x < 32) {
		uint32_t base = warp_lookback(w.lb_fin, chunk, total, epoch, &w.ctr->err);
		if (threadIdx.x == 0) s_base = base;
	}
	__syncthreads();
	uint32_t run = s_base + excl;
#pragma unroll
	for (uint32_t q = 0; q < KEEP; q++) {
		if (ta + q < tb) w.dbase[ta + q] = run;
		run += kept[q];
	}
	for (uint32_t tl = ta + KEEP; tl < tb; tl++) {
		w.dbase[tl] = run;
		run += tile_count(tl);
	}
	if (chunk == gridDim.x - 1 && threadIdx.x == 0) {
		const uint32_t n = s_base + total;
		w.dbase[w.n_tiles] = n;
		if (n > w.cap) atomicOr(&w.ctr->err, ERRF_OVERFLOW);
		if (!FUSED) w.ctr->n_agents = min(n, w.cap);
	}
	__threadfence();
	__syncthreads();
	if (threadIdx.x == 0) {
		s_last = 0;
		uint32_t done = atomicAdd(&w.ctr->finish_done, 1u);
		if (done == gridDim.x - 1) {
			__threadfence();
			s_last = 1;
			if (FUSED) {
				const uint32_t n = ld_volatile_u32(&w.ctr->n_all);
				if (n > w.cap) atomicOr(&w.ctr->err, ERRF_OVERFLOW);
				w.ctr->n_agents = min(n, w.cap);
				w.ctr->n_all = 0;
			}
			if (FULL) {
				w.ctr->giter = g;
				w.ctr->xtop = 0;
				for (int q = 0; q < 8; q++) w.ctr->sort_ticket[q] = 0;
			}
			w.ctr->seq = w.ctr->seq + 1;
			w.ctr->fin_ticket = 0;
			w.ctr->finish_done = 0;
		}
	}
	__syncthreads();
	if (FULL && s_last) {
		/* every run's row g is complete: fold it into its focal measures
		 * (read through L2: the row was summed by atomics) */
		for (uint32_t r = threadIdx.x; r < w.nruns_cap; r += blockDim.x) {
			const RunDev &run = w.runs[r];
			const uint32_t t = g - run.start_giter;
			if (!run_live(run, t)) continue;
			const PPStatistics *st = &w.ring[(size_t) (g % w.ring_rows) * w.nruns_cap + r];
			double o[6];
			focal_outputs(__ldcg(&st->sheep), __ldcg(&st->wolves), __ldcg(&st->grass),
				__ldcg((const unsigned long long *) &st->sheep_en),
				__ldcg((const unsigned long long *) &st->wolves_en),
				__ldcg((const unsigned long long *) &st->grass_en), run.ncells, o);
			focal_fold(w.focal[r], o, t, false, run.ss_from);
		}
		for (uint32_t q = threadIdx.x; q < 8 * 256; q += blockDim.x) w.hist[q] = 0;
		const uint32_t nrow = (g + 1) % w.ring_rows;
		uint32_t *rowp = reinterpret_cast<uint32_t *>(
			&w.ring[(size_t) nrow * w.nruns_cap]);
		const uint32_t words = w.nruns_cap * (sizeof(PPStatistics) / 4);
		for (uint32_t q = threadIdx.x; q < words; q += blockDim.x) rowp[q] = 0;
	}
}

__global__ void k_focal_init(WorldDev w, uint32_t r, uint32_t row, uint32_t t0)
{
	const PPStatistics *st = &w.ring[(size_t) row * w.nruns_cap + r];
	double o[6];
	focal_outputs(st->sheep, st->wolves, st->grass, st->sheep_en, st->wolves_en,
		st->grass_en, w.runs[r].ncells, o);
	focal_fold(w.focal[r], o, t0, true, w.runs[r].ss_from);
}

/* Regions of tiles [first, first + count) from the tile offsets of a
 * cell-sorted array placed at `base` of the region buffer. */
__global__ void k_regions_set(WorldDev w, uint32_t first, uint32_t count,
	uint32_t base)
{
	for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < count;
		q += gridDim.x * blockDim.x) {
		const uint32_t t = first + q;
		w.rstart[t] = base + w.tile_off[t];
		w.rcnt[t] = w.tile_off[t + 1] - w.tile_off[t];
	}
}

/* After a standalone sort on the world's counters (initial agents, an
 * admitted run): new look-back epochs, fresh sort tickets and histograms. */
__global__ void k_after_sort(WorldCounters *ctr, uint32_t *hist)
{
	for (uint32_t q = threadIdx.x; q < 8 * 256; q += blockDim.x) hist[q] = 0;
	if (threadIdx.x == 0) {
		ctr->seq = ctr->seq + 1;
		for (int q = 0; q < 8; q++) ctr->sort_ticket[q] = 0;
	}
}

/* ------------------------------------------------------------------ */
/* Init and stats of a freshly initialised run                         */
/* ------------------------------------------------------------------ */

/* Initial grass of a run: countdown c (0 = alive) stored as the regrowth
 * iteration c, c counted in the run's regrowth histogram (shared-memory
 * atomics, cheaper here than a ballot per value), and the live cells and
 * the countdown sum added to the run's stats row. */
__global__ void __launch_bounds__(ACT_THREADS) k_init_grass(WorldDev w, RunDev run,
	PPStatistics *dst)
{
	__shared__ uint32_t sh[1024];
	__shared__ uint64_t red[2][ACT_THREADS / 32];
	const uint32_t fs = run.restart + 1;
	const bool local = fs <= 1024;
	const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	if (local)
		for (uint32_t q = threadIdx.x; q < fs; q += blockDim.x) sh[q] = 0;
	__syncthreads();
	const uint32_t span = run.n_tiles << w.log_tile;
	uint32_t alive_n = 0;
	uint64_t csum = 0;
	for (uint32_t lc = blockIdx.x * blockDim.x + threadIdx.x; lc < span;
		lc += gridDim.x * blockDim.x) {
		uint32_t v = 0;
		if (lc < run.ncells) {
			u4 r = rng(run.seed_lo, run.seed_hi, lc, 0, STREAM_INIT_CELL, 0);
			uint32_t alive = draw(r.x, 2);
			v = alive ? 0 : 1 + draw(r.y, run.restart);
			alive_n += v == 0;
			csum += v;
		}
		w.grass[run.cbase + lc] = (uint16_t) v;
		if (v) {
			if (local) atomicAdd(&sh[v], 1u);
			else atomicAdd(&w.fring[run.fbase + v], 1u);
		}
	}
	const uint64_t a = warp_sum((uint64_t) alive_n), g = warp_sum(csum);
	if (lane == 0) {
		red[0][wid] = a;
		red[1][wid] = g;
	}
	__syncthreads();
	if (local)
		for (uint32_t q = threadIdx.x; q < fs; q += blockDim.x)
			if (sh[q]) atomicAdd(&w.fring[run.fbase + q], sh[q]);
	if (threadIdx.x < 2) {
		uint64_t sum = 0;
		for (uint32_t q = 0; q < ACT_THREADS / 32; q++) sum += red[threadIdx.x][q];
		stats_atomic_add(dst, threadIdx.x ? 5u : 2u, sum);
	}
}

/* Every alive cell's regrowth iteration moved to the run's current
 * iteration t (countdown 0 either way), so (int16)(regrowth - t) never
 * wraps: run every few thousand iterations. */
__global__ void k_grass_rebase(WorldDev w)
{
	const uint32_t gdone = w.ctr->giter;
	const uint32_t cells = w.n_tiles << w.log_tile;
	for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < cells;
		c += gridDim.x * blockDim.x) {
		const RunDev &run = w.runs[w.tile_run[c >> w.log_tile]];
		const uint32_t t = gdone - run.start_giter;
		if (!run.active || c - run.cbase >= run.ncells) continue;
		const uint16_t t16 = (uint16_t) t;
		const int32_t dd = (int16_t) (uint16_t) (w.grass[c] - t16);
		if (dd < 0) w.grass[c] = t16;
	}
}

/* Initial agents of a run, in creation order, into k/v[base ..); their
 * counts and energy sums added to the run's stats row. */
__global__ void __launch_bounds__(ACT_THREADS) k_init_agents(RunDev run,
	uint32_t *k, uint32_t *v, uint32_t base, uint32_t n_sheep, uint32_t n_wolves,
	PPStatistics *dst)
{
	__shared__ uint64_t s_part[6];
	StatAcc acc;
	acc.zero();
	const uint32_t n = n_sheep + n_wolves;
	for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < n;
		a += gridDim.x * blockDim.x) {
		u4 r = rng(run.seed_lo, run.seed_hi, a, 0, STREAM_INIT_AGENT, 0);
		uint32_t x = draw(r.x, run.gx), y = draw(r.y, run.gy);
		bool wolf = a >= n_sheep;
		uint32_t gain = wolf ? run.wolves_gain : run.sheep_gain;
		uint32_t e = (1 + draw(r.z, 2 * gain)) & run.emask;
		k[base + a] = run.cbase + y * run.gx + x;
		v[base + a] = (wolf ? TYPE_BIT : 0u) | e;
		if (wolf) { acc.wolves++; acc.wen += e; }
		else { acc.sheep++; acc.sen += e; }
	}
	block_stats(acc, s_part);
	if (threadIdx.x < 6) stats_atomic_add(dst, threadIdx.x, s_part[threadIdx.x]);
}

/* Initial agents bucketed by tile (fused pipeline): agents per tile, the
 * tiles' exclusive offsets, then each agent written into its tile's bucket
 * as one 16-byte record with its creation index. A bucket's order is that
 * of the atomics; the first move restores each cell's creation order from
 * the indices. */
__global__ void k_bucket_count(const uint32_t *k, uint32_t n, uint32_t log_tile,
	uint32_t *cnt)
{
	for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < n;
		a += gridDim.x * blockDim.x)
		atomicAdd(&cnt[k[a] >> log_tile], 1u);
}

/* Exclusive scan in place of off[first, first + count] (the last entry
 * enters as 0 and leaves as the total), copied to cursor[first, first +
 * count), in chunks of BSCAN_CHUNK entries: the chunks' sums, then every
 * chunk scanned from the sum of the chunks before it. */
constexpr uint32_t BSCAN_THREADS = 1024, BSCAN_CHUNK = 4 * BSCAN_THREADS;

__device__ __forceinline__ uint32_t bscan_block_excl(uint32_t x_in, uint32_t *ws,
	uint32_t *total)
{
	const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	uint32_t x = x_in;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
		if (lane >= (uint32_t) o) x += y;
	}
	if (lane == 31) ws[wid] = x;
	__syncthreads();
	if (wid == 0) {
		uint32_t y = ws[lane];
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const uint32_t z = __shfl_up_sync(0xffffffffu, y, o);
			if (lane >= (uint32_t) o) y += z;
		}
		ws[lane] = y;
	}
	__syncthreads();
	*total = ws[BSCAN_THREADS / 32 - 1];
	return (wid ? ws[wid - 1] : 0u) + x - x_in;
}

__global__ void __launch_bounds__(BSCAN_THREADS) k_bucket_sums(const uint32_t *off,
	uint32_t first, uint32_t count, uint32_t *part)
{
	__shared__ uint32_t ws[BSCAN_THREADS / 32];
	const uint32_t n = count + 1, c0 = blockIdx.x * BSCAN_CHUNK;
	uint32_t sum = 0;
#pragma unroll
	for (int q = 0; q < 4; q++) {
		const uint32_t i = c0 + q * BSCAN_THREADS + threadIdx.x;
		if (i < n) sum += off[first + i];
	}
	uint32_t total;
	bscan_block_excl(sum, ws, &total);
	if (threadIdx.x == 0) part[blockIdx.x] = total;
}

__global__ void __launch_bounds__(BSCAN_THREADS) k_bucket_scan(uint32_t *off,
	uint32_t *cursor, uint32_t first, uint32_t count, const uint32_t *part)
{
	__shared__ uint32_t ws[BSCAN_THREADS / 32];
	const uint32_t n = count + 1, c0 = blockIdx.x * BSCAN_CHUNK;
	/* the sum of the chunks before this one */
	uint32_t before = 0;
	for (uint32_t q = threadIdx.x; q < blockIdx.x; q += BSCAN_THREADS) before += part[q];
	uint32_t total;
	bscan_block_excl(before, ws, &total);
	const uint32_t prefix = total;
	__syncthreads();
	uint32_t v[4], sum = 0;
#pragma unroll
	for (int q = 0; q < 4; q++) {
		const uint32_t i = c0 + 4 * threadIdx.x + q;
		v[q] = i < n ? off[first + i] : 0u;
		sum += v[q];
	}
	uint32_t run = prefix + bscan_block_excl(sum, ws, &total);
#pragma unroll
	for (int q = 0; q < 4; q++) {
		const uint32_t i = c0 + 4 * threadIdx.x + q;
		if (i < n) {
			off[first + i] = run;
			if (i < count) cursor[first + i] = run;
		}
		run += v[q];
	}
}

__global__ void k_bucket_scatter(const uint32_t *k, const uint32_t *v, uint32_t n,
	uint32_t log_tile, uint32_t *cursor, uint4 *out)
{
	for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < n;
		a += gridDim.x * blockDim.x) {
		const uint32_t kk = k[a];
		const uint32_t pos = atomicAdd(&cursor[kk >> log_tile], 1u);
		out[pos] = make_uint4(kk, v[a], a, 0u);
	}
}

/* Self-test of the bounded look-back the finish kernel uses: one warp per
 * chunk (chunks taken by ticket, so a chunk's predecessors are running or
 * done) publishes chunk + 1 and looks back; chunk `stall` never publishes,
 * so the wait of the chunk after it runs out after `limit` polls and raises
 * ERRF_TIMEOUT instead of hanging. */
__global__ void k_lookback_selftest(uint64_t *lb, uint32_t *ticket, uint32_t *err,
	uint32_t *prefix, uint32_t stall, uint32_t limit)
{
	uint32_t chunk = 0;
	if (threadIdx.x == 0) chunk = atomicAdd(ticket, 1u);
	chunk = __shfl_sync(0xffffffffu, chunk, 0);
	if (chunk == stall) return;
	const uint32_t excl = warp_lookback(lb, chunk, chunk + 1, 1u, err, limit);
	if (threadIdx.x == 0) prefix[chunk] = excl;
}

__global__ void k_philox_fill(uint32_t c0, uint32_t c1, uint32_t c2,
	uint32_t c3, uint32_t k0, uint32_t k1, uint32_t n, uint32_t *out)
{
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
		i += gridDim.x * blockDim.x) {
		u4 r = philox4x32_10(u4{c0 + i, c1, c2, c3}, k0, k1);
		reinterpret_cast<uint4 *>(out)[i] = make_uint4(r.x, r.y, r.z, r.w);
	}
}

/* ------------------------------------------------------------------ */
/* Host-side launch wrappers                                           */
/* ------------------------------------------------------------------ */

cudaError_t enqueue_iteration(const WorldDev &w, const LaunchCfg &lc,
	cudaStream_t s, const cudaEvent_t *marks)
{
	/* marks (optional, passes + 5 events): before the move, after the
	 * move, after each radix pass, after the offsets, after the act, after
	 * the finish. */
	if (marks) cudaEventRecord(marks[0], s);
	size_t hist_smem = (size_t) (w.passes << w.digit_bits) * sizeof(uint32_t);
	k_regions<true><<<lc.move_blocks, 256, hist_smem, s>>>(w, w.kB, w.vB);
	if (marks) cudaEventRecord(marks[1], s);
	uint32_t *ki = w.kB, *vi = w.vB, *ko = w.kC, *vo = w.vC;
	for (uint32_t p = 0; p < w.passes; p++) {
		cudaError_t e = launch_radix_pass(ki, vi, ko, vo, w.hist + p * 256,
			w.lb_sort, w.ctr, &w.ctr->n_agents, p, w.sort_shift + p * w.digit_bits,
			w.digit_bits, lc.sort_blocks, s);
		if (e != cudaSuccess) return e;
		if (marks) cudaEventRecord(marks[2 + p], s);
		uint32_t *tk = ki, *tv = vi;
		ki = ko; vi = vo; ko = tk; vo = tv;
	}
	/* ki/vi now hold the cell-sorted agents (dead ones last). */
	k_offsets<<<lc.offs_blocks, 256, 0, s>>>(ki, &w.ctr->n_agents,
		w.log_tile, w.n_tiles, w.tile_off);
	if (marks) cudaEventRecord(marks[2 + w.passes], s);
	size_t act_smem = (size_t) w.act_cap * 5 * sizeof(uint32_t)
		+ ((size_t) lc.cpt * ACT_THREADS) * sizeof(uint32_t);
	/* (the shared-memory layout of k_act: five agent arrays, then the
	 * tile's per-cell counters) */
	switch (lc.cpt) {
	case 4: k_act<4><<<w.n_tiles, ACT_THREADS, act_smem, s>>>(w, ki, vi); break;
	case 16: k_act<16><<<w.n_tiles, ACT_THREADS, act_smem, s>>>(w, ki, vi); break;
	case 32: k_act<32><<<w.n_tiles, ACT_THREADS, act_smem, s>>>(w, ki, vi); break;
	default: k_act<8><<<w.n_tiles, ACT_THREADS, act_smem, s>>>(w, ki, vi); break;
	}
	if (marks) cudaEventRecord(marks[3 + w.passes], s);
	k_finish<true, false><<<lc.finish_blocks, 256, 0, s>>>(w);
	if (marks) cudaEventRecord(marks[4 + w.passes], s);
	return cudaGetLastError();
}

cudaError_t launch_finish_fused(const WorldDev &w, const LaunchCfg &lc,
	cudaStream_t s)
{
	k_finish<true, true><<<lc.finish_blocks, 256, 0, s>>>(w);
	return cudaGetLastError();
}

cudaError_t enqueue_fused_bases(const WorldDev &w, const LaunchCfg &lc,
	cudaStream_t s)
{
	k_finish<false, true><<<lc.finish_blocks, 256, 0, s>>>(w);
	return cudaGetLastError();
}

cudaError_t set_act_smem_limits(size_t bytes)
{
	cudaError_t e;
	e = cudaFuncSetAttribute(k_act<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) bytes);
	if (e != cudaSuccess) return e;
	e = cudaFuncSetAttribute(k_act<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) bytes);
	if (e != cudaSuccess) return e;
	e = cudaFuncSetAttribute(k_act<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) bytes);
	if (e != cudaSuccess) return e;
	return cudaFuncSetAttribute(k_act<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) bytes);
}

cudaError_t enqueue_focal_init(const WorldDev &w, uint32_t r, uint32_t row,
	uint32_t t0, cudaStream_t s)
{
	k_focal_init<<<1, 1, 0, s>>>(w, r, row, t0);
	return cudaGetLastError();
}

cudaError_t enqueue_init_grass(const WorldDev &w, const RunDev &run,
	uint32_t r, uint32_t row, cudaStream_t s)
{
	uint32_t span = run.n_tiles << w.log_tile;
	uint32_t gb = (span + ACT_THREADS - 1) / ACT_THREADS;
	if (gb > 4096) gb = 4096;
	if (gb == 0) gb = 1;
	k_init_grass<<<gb, ACT_THREADS, 0, s>>>(w, run,
		&w.ring[(size_t) row * w.nruns_cap + r]);
	return cudaGetLastError();
}

cudaError_t enqueue_init_agents(const WorldDev &w, const RunDev &run,
	uint32_t r, uint32_t row, uint32_t *k, uint32_t *v, uint32_t base,
	uint32_t init_sheep, uint32_t init_wolves, cudaStream_t s)
{
	uint32_t n = init_sheep + init_wolves;
	if (!n) return cudaSuccess;
	uint32_t ab = (n + ACT_THREADS - 1) / ACT_THREADS;
	if (ab > 4096) ab = 4096;
	k_init_agents<<<ab, ACT_THREADS, 0, s>>>(run, k, v, base, init_sheep, init_wolves,
		&w.ring[(size_t) row * w.nruns_cap + r]);
	return cudaGetLastError();
}

cudaError_t enqueue_bucket_agents(const WorldDev &w, uint32_t n,
	uint32_t first, uint32_t count, cudaStream_t s)
{
	/* the fused pipeline does not use the region counters: they serve as
	 * the buckets' fill cursors */
	const uint32_t b = std::max<uint32_t>(1, std::min<uint32_t>((n + 255) / 256, 4096));
	const uint32_t chunks = (count + 1 + BSCAN_CHUNK - 1) / BSCAN_CHUNK;
	if (n) k_bucket_count<<<b, 256, 0, s>>>(w.kB, n, w.log_tile, w.tile_off);
	k_bucket_sums<<<chunks, BSCAN_THREADS, 0, s>>>(w.tile_off, first, count, w.bscan);
	k_bucket_scan<<<chunks, BSCAN_THREADS, 0, s>>>(w.tile_off, w.rcnt, first, count,
		w.bscan);
	if (n) k_bucket_scatter<<<b, 256, 0, s>>>(w.kB, w.vB, n, w.log_tile, w.rcnt,
		w.bucket);
	return cudaGetLastError();
}

cudaError_t launch_lookback_selftest(uint64_t *lb, uint32_t *ticket, uint32_t *err,
	uint32_t *prefix, uint32_t n, uint32_t stall, uint32_t limit, cudaStream_t s)
{
	k_lookback_selftest<<<n, 32, 0, s>>>(lb, ticket, err, prefix, stall, limit);
	return cudaGetLastError();
}

cudaError_t enqueue_regions_from_sorted(const WorldDev &w, const LaunchCfg &lc,
	const uint32_t *sorted_keys, uint32_t first, uint32_t count,
	uint32_t base, cudaStream_t s)
{
	/* tile offsets of the sorted agents (count from ctr->aux_n), regions of
	 * the given tiles, then dense bases of all regions */
	k_offsets<<<lc.offs_blocks, 256, 0, s>>>(sorted_keys, &w.ctr->aux_n,
		w.log_tile, w.n_tiles, w.tile_off);
	uint32_t b = (count + 255) / 256;
	if (b == 0) b = 1;
	if (b > 4096) b = 4096;
	k_regions_set<<<b, 256, 0, s>>>(w, first, count, base);
	k_finish<false, false><<<lc.finish_blocks, 256, 0, s>>>(w);
	return cudaGetLastError();
}

cudaError_t enqueue_compact(const WorldDev &w, const LaunchCfg &lc,
	uint32_t *ko, uint32_t *vo, cudaStream_t s)
{
	k_regions<false><<<lc.move_blocks, 256, 0, s>>>(w, ko, vo);
	return cudaGetLastError();
}

cudaError_t enqueue_grass_rebase(const WorldDev &w, const LaunchCfg &lc,
	cudaStream_t s)
{
	k_grass_rebase<<<lc.sms * 8, 256, 0, s>>>(w);
	return cudaGetLastError();
}

cudaError_t enqueue_after_sort(WorldCounters *ctr, uint32_t *hist,
	cudaStream_t s)
{
	k_after_sort<<<1, 256, 0, s>>>(ctr, hist);
	return cudaGetLastError();
}

cudaError_t launch_move_only(const uint32_t *kin, const uint32_t *vin,
	uint32_t *kout, uint32_t *vout, uint32_t n, const RunDev *run_dev,
	uint32_t iter, uint32_t dead_key, cudaStream_t s)
{
	uint32_t b = (n + 255) / 256;
	if (b > 4096) b = 4096;
	if (b == 0) b = 1;
	k_move_only<<<b, 256, 0, s>>>(kin, vin, kout, vout, n, run_dev, iter,
		dead_key);
	return cudaGetLastError();
}

cudaError_t launch_offsets(const uint32_t *keys, const uint32_t *n_dev,
	uint32_t log_tile, uint32_t n_buckets, uint32_t *off, int blocks,
	cudaStream_t s)
{
	k_offsets<<<blocks, 256, 0, s>>>(keys, n_dev, log_tile, n_buckets, off);
	return cudaGetLastError();
}

cudaError_t launch_philox_fill(uint32_t c0, uint32_t c1, uint32_t c2,
	uint32_t c3, uint32_t k0, uint32_t k1, uint32_t n, uint32_t *out,
	cudaStream_t s)
{
	uint32_t b = (n + 255) / 256;
	if (b > 4096) b = 4096;
	if (b == 0) b = 1;
	k_philox_fill<<<b, 256, 0, s>>>(c0, c1, c2, c3, k0, k1, n, out);
	return cudaGetLastError();
}

int occupancy_act(int cpt, size_t smem)
{
	int n = 0;
	cudaError_t e;
	switch (cpt) {
	case 4: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_act<4>, ACT_THREADS, smem); break;
	case 16: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_act<16>, ACT_THREADS, smem); break;
	case 32: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_act<32>, ACT_THREADS, smem); break;
	default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_act<8>, ACT_THREADS, smem); break;
	}
	if (e != cudaSuccess) { cudaGetLastError(); return 1; }
	return n;
}

} /* namespace pp */
