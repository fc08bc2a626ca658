/*
 * pp_fused.cu -- the fused iteration: one kernel per iteration does the
 * act of iteration t and the move of iteration t + 1 (opencl/pp/pp_gpu.cl
 * action_agent 883-979 followed by move_agent 744-821), so no sort runs
 * between the two.
 *
 * State between iterations (per parity of the world iteration):
 *   group buffer  records of moved agents (pp_device.cuh), written by the
 *                 act of each source tile as one contiguous group per
 *                 destination tile it sends to (plus one group of dead and
 *                 parked records), at twice the tile's dense input base;
 *   inboxes       per destination tile, up to IBX {start, count} entries
 *                 naming the groups destined to it.
 * The act of a tile gathers its groups, groups its agents by cell (counting
 * sort in shared memory), puts each cell's list in canonical order (source
 * cell, rank in the source cell's list: both are in the record), runs the
 * cells' actions exactly as the sort pipeline does, and then moves every
 * survivor and newborn: the move draw is keyed by (cell, t + 1, MOVE, rank
 * in the cell's new list), which the act knows. Positions inside a group
 * are arbitrary, because the next act orders each cell's list by the
 * record's (source cell, rank) and not by position. The finish kernel
 * sums each tile's posted group sizes into the dense input bases of the
 * next act, so no act allocates with an atomic on a shared counter.
 */
#include <algorithm>
#include <type_traits>

#include "pp_act.cuh"

namespace pp {

cudaError_t launch_finish_fused(const WorldDev &w, const LaunchCfg &lc,
	cudaStream_t s);

namespace {

static_assert(IBX == 32, "the inbox is read by one warp");

/* Threads per tile CTA: 128 for sparse tiles (nine CTAs per SM) and for
 * 512-cell tiles, 256 when a tile of 1024 cells or more may hold more
 * agents than half its cells (its shared memory then limits the SM to about
 * four CTAs). */
constexpr int NT_SPARSE = 128, NT_DENSE = 256;
/* Resident CTAs per SM the register allocation is bounded for: 56
 * registers a thread for 128-thread CTAs (nine per SM; 48 registers, ten
 * per SM, spill and run slower), 64 for 256-thread ones. */
#define CTAS_PER_SM(nt) ((nt) == NT_SPARSE ? 9 : 4)
constexpr uint32_t NCLS = 32;          /* group classes of a tile (one per lane) */
constexpr uint32_t CLS_FOREIGN = 30;   /* classes 0..29: other destination tiles */
constexpr uint32_t CLS_OWN = 30;       /* moved within the tile                  */
constexpr uint32_t CLS_GRAVE = 31;     /* dead and parked records                */
constexpr uint32_t CLS_NONE = 0xffffffffu;   /* table full: record dropped (error) */
/* direction code of a dropped output in the move phase's record cache (no
 * record carries it: records use 0-4, DIR_PARKED and DIR_DEAD) */
constexpr uint32_t DIR_DROPPED = 5;
static_assert(DIR_DROPPED != DIR_PARKED && DIR_DROPPED != DIR_DEAD, "cache code");
constexpr uint32_t TBL_EMPTY = 0xffffffffu;

/* Class of destination tile dt (not the CTA's own tile) in the CTA's table
 * of destination tiles, inserted when new; CLS_NONE if the table is full
 * (a tile sends to at most 15 other tiles, so this does not happen). */
__device__ __forceinline__ uint32_t class_insert(uint32_t *tbl, uint32_t dt)
{
	uint32_t h = dt % CLS_FOREIGN;
	for (uint32_t p = 0; p < CLS_FOREIGN; p++) {
		uint32_t cur = *(volatile uint32_t *) &tbl[h];
		if (cur == dt) return h;
		if (cur == TBL_EMPTY) {
			cur = atomicCAS(&tbl[h], TBL_EMPTY, dt);
			if (cur == TBL_EMPTY || cur == dt) return h;
		}
		h = (h + 1 == CLS_FOREIGN) ? 0 : h + 1;
	}
	return CLS_NONE;
}

__device__ __forceinline__ uint32_t class_find(const uint32_t *tbl, uint32_t dt)
{
	uint32_t h = dt % CLS_FOREIGN;
	for (uint32_t p = 0; p < CLS_FOREIGN; p++) {
		if (tbl[h] == dt) return h;
		h = (h + 1 == CLS_FOREIGN) ? 0 : h + 1;
	}
	return CLS_NONE;
}

/* 16-byte asynchronous copy global -> shared (cp.async, bypassing L1). */
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
	const uint32_t sa = (uint32_t) __cvta_generic_to_shared(smem);
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16;"
		:: "r"(sa), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_commit()
{
	asm volatile("cp.async.commit_group;" ::: "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
	asm volatile("cp.async.wait_group 0;" ::: "memory");
}

/* ctr[key] += 1 for every calling lane, one atomic per distinct key per
 * warp; returns the counter's value before this lane's increment. */
__device__ __forceinline__ uint32_t warp_agg_add(uint32_t *ctr, uint32_t key)
{
	const uint32_t act = __activemask();
	const uint32_t peers = __match_any_sync(act, key);
	const uint32_t lane = threadIdx.x & 31;
	const uint32_t leader = __ffs(peers) - 1;
	uint32_t base = 0;
	if (lane == leader) base = atomicAdd(&ctr[key], (uint32_t) __popc(peers));
	base = __shfl_sync(peers, base, leader);
	return base + __popc(peers & ((1u << lane) - 1));
}

/* Exclusive scan of one value per thread over the NT threads of the CTA;
 * the total goes to *total. */
template <int NT>
__device__ __forceinline__ uint32_t step_excl_scan(uint32_t v, uint32_t *total)
{
	__shared__ uint32_t ws[NT / 32];
	const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	uint32_t x = v;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
		if (lane >= (uint32_t) o) x += y;
	}
	if (lane == 31) ws[wid] = x;
	__syncthreads();
	uint32_t before = 0, all = 0;
#pragma unroll
	for (uint32_t q = 0; q < NT / 32; q++) {
		const uint32_t c = ws[q];
		if (q < wid) before += c;
		all += c;
	}
	*total = all;
	__syncthreads();
	return before + x - v;
}

/* One CTA of NT threads per tile of CPT * NT cells.
 *   ACT:  the act of iteration t of the tile's agents (gathered from its
 *         inbox of parity t) and the move of iteration t + 1 of its
 *         survivors and newborns into the group buffer of parity t + 1.
 *   !ACT: the move of iteration 1 of a freshly initialised run's agents,
 *         read from w.bucket at the tile offsets, where they lie in no
 *         particular order with their creation indices (a cell's list is
 *         its agents in creation order).
 * Phases (ACT): gather; counting sort by cell, each agent of a multi-agent
 * cell placed by its rank in canonical order; B draws; C actions, one
 * thread per agent (as the sort pipeline's act); E0 output offsets and
 * stats; E1 move draws and per-class counts;
 * one warp allocates the tile's groups and posts them to the destination
 * tiles' inboxes; E2 records into the groups; per-tile stats. (!ACT: the
 * bucket read and counted per cell, the same counting sort with each
 * cell's agents in creation order, then E1 and E2 on every agent.) */
template <int CPT, int NT, bool ACT>
__device__ __forceinline__ void step_tile(const WorldDev &w, uint32_t tile,
	uint32_t out_base, uint32_t *sm)
{
	uint32_t *sk = sm, *sv = sm + w.act_cap, *sp = sv + w.act_cap,
		*sd = sp + w.act_cap, *sperm = sd + w.act_cap;
	uint32_t *scnt = sperm + w.act_cap;                 /* CPT * NT */
	uint16_t *sgrass = reinterpret_cast<uint16_t *>(scnt + CPT * NT);
	__shared__ uint32_t s_tbl[CLS_FOREIGN];
	__shared__ uint32_t s_ccnt[NCLS + 1], s_cpos[NCLS + 1];   /* + a discard slot */
	__shared__ uint32_t s_xbase, s_fail;
	__shared__ uint64_t red[5][NT / 32];    /* per-warp partial stats */

	const uint32_t tid = threadIdx.x, lane = tid & 31;
	const uint32_t c0 = tile << w.log_tile;
	/* loads that depend on nothing, issued first: the tile's grass (async
	 * copy into shared memory), both parities' inboxes (every warp reads
	 * its own copy: no barrier before the gather), the tile's dense input
	 * base */
	uint32_t in_n0 = 0, in_n1 = 0, dbase_t = 0;
	uint2 in_e0 = make_uint2(0u, 0u), in_e1 = make_uint2(0u, 0u);
	if (ACT) {
		const uint4 *src = reinterpret_cast<const uint4 *>(w.grass + c0);
		for (uint32_t q = tid; q < CPT * NT / 8; q += NT)
			cp_async16(reinterpret_cast<uint4 *>(sgrass) + q, src + q);
		cp_async_commit();
		const size_t ib0 = tile, ib1 = (size_t) w.n_tiles + tile;
		in_n0 = w.inbox_n[ib0];
		in_n1 = w.inbox_n[ib1];
		in_e0 = w.inbox[ib0 * IBX + lane];
		in_e1 = w.inbox[ib1 * IBX + lane];
		dbase_t = w.dbase[tile];
	}
	const uint32_t g = w.ctr->giter + 1;
	const uint32_t err_now = ACT ? w.ctr->err : 0u;
	const uint32_t pin = g & 1, pout = ACT ? (g + 1) & 1 : g & 1;
	/* the run's parameters, copied to shared memory: they are read in every
	 * phase, and through a reference into global memory they would be
	 * reloaded after each global store (the compiler cannot rule out
	 * aliasing) */
	__shared__ RunDev s_run;
	const RunDev &grun = w.runs[w.tile_run[tile]];
	static_assert(sizeof(RunDev) % 4 == 0 && sizeof(RunDev) / 4 <= NT, "run copy");
	if (tid < sizeof(RunDev) / 4)
		reinterpret_cast<uint32_t *>(&s_run)[tid] = reinterpret_cast<const uint32_t *>(&grun)[tid];
	const RunDev &run = s_run;
	const uint32_t t = g - grun.start_giter;
	/* a world whose agent pool has overflowed is failed (the host returns
	 * PP_OUT_OF_RESOURCES at its next check): its later acts do nothing,
	 * so a run that overflowed early does not grind through its remaining
	 * iterations on a corrupted state */
	if (ACT && (!run_live(grun, t) || (err_now & ERRF_OVERFLOW))) {
		cp_async_wait_all();
		/* finished run, free tile space or a failed world: nothing
		 * survives, no stats */
		if (tid == 0) w.inbox_n[(size_t) pin * w.n_tiles + tile] = 0;
		if (tid < 8) w.part[(size_t) tile * 8 + tid] = 0;
		return;
	}
	const uint32_t tmove = ACT ? t + 1 : t;
	const bool live_move = run_live(grun, tmove);
	const uint32_t seed_lo = grun.seed_lo, seed_hi = grun.seed_hi;
	const uint32_t lt0 = c0 - grun.cbase;         /* run-local index of the tile start */
	const uint32_t lcmask = (1u << w.log_tile) - 1;
	if (tid < CLS_FOREIGN) s_tbl[tid] = TBL_EMPTY;
	if (tid <= NCLS) s_ccnt[tid] = 0;
	if (tid == NCLS) s_cpos[NCLS] = 0;
	/* per-cell counters, transposed in groups of four: thread k's cells
	 * k CPT + 4 a .. + 3 are the 16 bytes at word 4 (a NT + k), so a warp
	 * reads its threads' counters with conflict-free 16-byte loads */
#define SLOT(c) (((((c) % CPT) >> 2) * NT + (c) / CPT) * 4 + ((c) & 3))
	{
		uint4 *z = reinterpret_cast<uint4 *>(scnt);
#pragma unroll
		for (int q = 0; q < CPT / 4; q++) z[q * NT + tid] = make_uint4(0u, 0u, 0u, 0u);
	}

	/* ---- inputs ---- */
	uint32_t m, a0 = 0;
	uint32_t grp_start = 0, grp_pref = 0, nin = 0;   /* this lane's inbox group */
	if (ACT) {
		/* entries past the count are stale and ignored */
		nin = min(pin ? in_n1 : in_n0, IBX);
		uint2 e = pin ? in_e1 : in_e0;
		if (lane >= nin) e = make_uint2(0u, 0u);
		const uint32_t c = (e.y & GROUP_GRAVE) ? 0u : e.y;
		uint32_t x = c;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
			if (lane >= (uint32_t) o) x += y;
		}
		grp_start = e.x;
		grp_pref = x - c;
		m = __shfl_sync(0xffffffffu, x, 31);
	} else {
		a0 = w.tile_off[tile];
		m = w.tile_off[tile + 1] - a0;
	}
	const bool in_smem = m <= w.act_cap;
	if (!in_smem) {
		/* crowded tile: its arrays go to global scratch (m slots of each
		 * array; 3 m of the permutation array, which then holds the output
		 * map and the move directions) */
		if (tid == 0) {
			const uint32_t b = atomicAdd(&w.ctr->xtop, m);
			s_fail = (uint64_t) b + m > w.cap;
			if (s_fail) atomicOr(&w.ctr->err, ERRF_OVERFLOW);
			s_xbase = b;
		}
	}
	__syncthreads();
	if (!in_smem && s_fail) {
		/* the tile's agents are dropped (the overflow is flagged): its
		 * inbox is emptied as if it had been read, so no later act reads
		 * these groups again */
		if (ACT) {
			cp_async_wait_all();
			if (tid == 0) w.inbox_n[(size_t) pin * w.n_tiles + tile] = 0;
		}
		if (tid < 8) w.part[(size_t) tile * 8 + tid] = 0;
		return;
	}
	/* The phases, instantiated once for a tile whose arrays are in shared
	 * memory and once for a crowded tile's global scratch: each copy then
	 * addresses one memory space directly (shared loads and stores with
	 * 32-bit addresses) instead of through generic pointers. */
	auto phases = [&](auto smem_tag, auto split_tag, uint32_t *UK, uint32_t *UV, uint32_t *PERM,
		uint32_t *LK, uint32_t *LV) {
		constexpr bool in_smem = decltype(smem_tag)::value;
		/* the move phase's record cache spread over the dead counter and
		 * grass words and the permutation array's tail (tiles whose 2 act_cap
		 * outputs do not fit the counters) */
		constexpr bool split = decltype(split_tag)::value;
		uint32_t *LP = UK, *LD = UV;      /* priorities / dice, then offsets / kids */

		uint32_t eats = 0;
		if (!ACT) {
			/* the tile's agents, counted per cell */
			for (uint32_t j = tid; j < m; j += NT) {
				const uint4 r = w.bucket[a0 + j];
				const uint32_t kk = r.x - c0;
				UK[j] = kk;
				UV[j] = r.y;
				atomicAdd(&scnt[SLOT(kk)], 1u);
			}
		} else {
			/* gather the tile's groups and count agents per cell: item j comes
			 * from the last group whose prefix is <= j (groups with equal
			 * prefixes before it are empty), found by a binary search over
			 * the lanes' group prefixes; two items in flight per thread */
			const uint32_t *kGi = pin ? w.kG1 : w.kG0;
			const uint32_t *vGi = pin ? w.vG1 : w.vG0;
			const uint32_t m_up = (m + NT - 1) / NT * NT;   /* warp-uniform trip count */
			if (m <= NT) {
				/* one item per thread: one group search instead of two */
				const uint32_t j = tid;
				uint32_t lo = 0, hi = max(nin, 1u);
#pragma unroll
				for (int step = 0; step < 5; step++) {
					const uint32_t mid = (lo + hi) >> 1;
					const uint32_t pm = __shfl_sync(0xffffffffu, grp_pref, mid);
					if (hi - lo > 1) {
						if (pm <= j) lo = mid; else hi = mid;
					}
				}
				const uint32_t src = __shfl_sync(0xffffffffu, grp_start, lo)
					+ (j - __shfl_sync(0xffffffffu, grp_pref, lo));
				if (j < m) {
					const uint32_t kk = kGi[src], vv = vGi[src];
					UK[j] = kk;
					UV[j] = vv;
					atomicAdd(&scnt[SLOT(kk & lcmask)], 1u);
				}
			} else
			for (uint32_t j0 = tid; j0 < m_up; j0 += 2 * NT) {
				uint32_t src[2];
#pragma unroll
				for (int u = 0; u < 2; u++) {
					const uint32_t j = j0 + u * NT;
					uint32_t lo = 0, hi = max(nin, 1u);     /* last q with pref <= j */
#pragma unroll
					for (int step = 0; step < 5; step++) {
						const uint32_t mid = (lo + hi) >> 1;
						const uint32_t pm = __shfl_sync(0xffffffffu, grp_pref, mid);
						if (hi - lo > 1) {
							if (pm <= j) lo = mid; else hi = mid;
						}
					}
					src[u] = __shfl_sync(0xffffffffu, grp_start, lo)
						+ (j - __shfl_sync(0xffffffffu, grp_pref, lo));
				}
				uint32_t kk[2], vv[2];
#pragma unroll
				for (int u = 0; u < 2; u++) {
					if (j0 + u * NT < m) {
						kk[u] = kGi[src[u]];
						vv[u] = vGi[src[u]];
					}
				}
#pragma unroll
				for (int u = 0; u < 2; u++) {
					const uint32_t j = j0 + u * NT;
					if (j < m) {
						UK[j] = kk[u];
						UV[j] = vv[u];
						atomicAdd(&scnt[SLOT(kk[u] & lcmask)], 1u);
					}
				}
			}
		}
		__syncthreads();
		if (ACT && tid == 0) w.inbox_n[(size_t) pin * w.n_tiles + tile] = 0;
		{
			uint4 *s4 = reinterpret_cast<uint4 *>(scnt);
			uint32_t loc = 0;
#pragma unroll
			for (int a = 0; a < CPT / 4; a++) {
				const uint4 v = s4[a * NT + tid];
				loc += v.x + v.y + v.z + v.w;
			}
			uint32_t tot;
			uint32_t run_start = step_excl_scan<NT>(loc, &tot);
#pragma unroll
			for (int a = 0; a < CPT / 4; a++) {
				const uint4 v = s4[a * NT + tid];
				uint4 o;
				o.x = run_start;
				o.y = o.x + v.x;
				o.z = o.y + v.y;
				o.w = o.z + v.z;
				run_start = o.w + v.w;
				s4[a * NT + tid] = o;
			}
		}
		__syncthreads();
		for (uint32_t j = tid; j < m; j += NT)
			PERM[atomicAdd(&scnt[SLOT(UK[j] & lcmask)], 1u)] = j;
		__syncthreads();
		/* scnt[SLOT(c)] is now the end of cell c, and cell c's agents
		 * occupy [end of c - 1, end of c) in arrival order; each goes to
		 * the cell's start plus its rank in canonical order, which only
		 * an agent sharing its cell has to count. Equal keys, which a
		 * consistent state never holds, are ordered by arrival, so the
		 * slots stay a permutation whatever the input (after an overflow,
		 * say). LK holds the cell in bits 0-15 and the rank in the cell's
		 * list in bits 16-31. */
		for (uint32_t i = tid; i < m; i += NT) {
			const uint32_t j = PERM[i];
			const uint32_t rk = UK[j], c = rk & lcmask;
			const uint32_t e = scnt[SLOT(c)], b = c ? scnt[SLOT(c - 1)] : 0;
			uint32_t d = i;
			if (e - b > 1) {
				if (ACT) {
					const uint32_t lr = lt0 + c;
					const uint32_t y = fastdiv_div(lr, run.gxdiv), x = lr - y * run.gx;
					/* the cell's four neighbour offsets, then each mate's
					 * key (source cell offset, rank in the source list)
					 * with selects rather than a switch on its arrival
					 * direction, so the lanes of a warp do not diverge */
					const int32_t o1 = src_offset(1, x, y, run.gx, run.gy);
					const int32_t o2 = src_offset(2, x, y, run.gx, run.gy);
					const int32_t o3 = src_offset(3, x, y, run.gx, run.gy);
					const int32_t o4 = src_offset(4, x, y, run.gx, run.gy);
					auto okey = [&](uint32_t rec) {
						const uint32_t dr = (rec >> REC_DIR_SHIFT) & 7u;
						const int32_t off = dr == 1 ? o1 : dr == 2 ? o2 : dr == 3 ? o3
							: dr == 4 ? o4 : 0;
						return (int64_t) off * 65536 + (rec >> REC_RANK_SHIFT);
					};
					const int64_t kx = okey(rk);
					d = b;
					for (uint32_t q = b; q < e; q++) {
						const uint32_t jq = PERM[q];
						const int64_t kq = okey(UK[jq]);
						d += kq < kx || (kq == kx && jq < j);
					}
				} else {
					/* initial agents: creation order */
					const uint32_t kx = w.bucket[a0 + j].z;
					d = b;
					for (uint32_t q = b; q < e; q++) {
						const uint32_t jq = PERM[q], kq = w.bucket[a0 + jq].z;
						d += kq < kx || (kq == kx && jq < j);
					}
				}
			}
			if (d - b > 0xffffu) atomicOr(&w.ctr->err, ERRF_OVERFLOW);
			LK[d] = c | (d - b) << 16;
			LV[d] = UV[j];
		}
		__syncthreads();
		if (ACT) {
			/* B: draws of every agent */
			for (uint32_t j = tid; j < m; j += NT) {
				const uint32_t lk = LK[j], lc = lk & 0xffffu;
				u4 r = rng(seed_lo, seed_hi, lt0 + lc, t, STREAM_ACT, lk >> 16);
				LP[j] = r.x;
				LD[j] = draw(r.y, 100);
			}
			cp_async_wait_all();
			__syncthreads();
			/* C: actions, one thread per agent */
			ActParams ap;
			ap.sheep_gain = run.sheep_gain; ap.sheep_thr = run.sheep_thr;
			ap.sheep_prob = run.sheep_prob; ap.wolves_gain = run.wolves_gain;
			ap.wolves_thr = run.wolves_thr; ap.wolves_prob = run.wolves_prob;
			ap.restart = run.restart;
			ap.emask = run.emask;
			const uint16_t t16 = (uint16_t) t;
			for (uint32_t j = tid; j < m; j += NT) {
				const uint32_t lk = LK[j], lc = lk & 0xffffu;
				/* the cell's agents are [p, e): the counters hold each
				 * cell's end since the copy into cell order */
				const uint32_t p = j - (lk >> 16);
				const uint32_t e = scnt[SLOT(lc)];
				const int32_t dd = (int16_t) (uint16_t) (sgrass[lc] - t16);
				uint32_t kid;
				if (act_agent(j, p, e, LV, LP, ap, dd > 0 ? (uint32_t) dd : 0u, LD[j], &kid)) {
					w.grass[c0 + lc] = (uint16_t) (t16 + (uint16_t) ap.restart);
					eats++;
				}
				LD[j] = kid;
			}
			__syncthreads();
		}

#undef SLOT
		/* ---- E0: output offsets (each survivor, then its newborn), stats,
		 * and the output -> agent map OUTJ (agent index | newborn << 15) ---- */
		const uint32_t ch = (m + NT - 1) / NT;
		const uint32_t ja = min(tid * ch, m), jb = min(ja + ch, m);
		uint32_t cnt = 0, sheep = 0, wolves = 0;
		uint64_t sen = 0, wen = 0;
		if (ACT) {
			for (uint32_t j = ja; j < jb; j++) {
				const uint32_t v = LV[j], kd = LD[j];
				const uint32_t tb = v & TYPE_BIT, en = v & ENERGY_MASK;
				if (!(v & EATEN_BIT)) {
					cnt++;
					if (tb) { wolves++; wen += en; } else { sheep++; sen += en; }
				}
				if (kd & KID_BIT) {
					cnt++;
					const uint32_t ke = kd & KID_ENERGY;
					if (tb) { wolves++; wen += ke; } else { sheep++; sen += ke; }
				}
			}
		}
		uint32_t total = m;
		/* output map: 16-bit entries in the permutation's shared array (2 m
		 * <= 2 act_cap), 32-bit ones in a crowded tile's scratch; directions:
		 * bytes in the cell counters (2 m <= 4 T) or after the map */
		uint16_t *OUTJ16 = reinterpret_cast<uint16_t *>(PERM);
		uint32_t *OUTJ32 = PERM;
		uint8_t *DIR = in_smem ? reinterpret_cast<uint8_t *>(scnt)
			: reinterpret_cast<uint8_t *>(PERM + 2 * m);
		if (ACT) {
			uint32_t o = step_excl_scan<NT>(cnt, &total);
			for (uint32_t j = ja; j < jb; j++) {
				LP[j] = o;
				if (!(LV[j] & EATEN_BIT)) {
					if (in_smem) OUTJ16[o] = (uint16_t) j; else OUTJ32[o] = j;
					o++;
				}
				if (LD[j] & KID_BIT) {
					if (in_smem) OUTJ16[o] = (uint16_t) (j | 0x8000u);
					else OUTJ32[o] = j | 0x80000000u;
					o++;
				}
			}
			__syncthreads();
		}
		/* the tile's slots in the group buffer: twice its dense input base
		 * (at most two outputs per input), or after out_base for a first move */
		const uint32_t gb = ACT ? 2 * dbase_t : out_base + a0;

		/* output o: its agent j, whether it is a newborn, its energy and rank
		 * in its cell's new list */
		auto output = [&](uint32_t o, uint32_t &j, uint32_t &nb, uint32_t &en,
			uint32_t &rank) {
			if (ACT) {
				if (in_smem) {
					const uint32_t u = OUTJ16[o];
					j = u & 0x7fffu;
					nb = u >> 15;
				} else {
					const uint32_t u = OUTJ32[o];
					j = u & 0x7fffffffu;
					nb = u >> 31;
				}
			} else {
				j = o;
				nb = 0;
			}
			const uint32_t lk = LK[j];
			const uint32_t f = j - (lk >> 16);
			rank = ACT ? o - LP[f] : lk >> 16;
			en = nb ? (LD[j] & KID_ENERGY) : (LV[j] & ENERGY_MASK);
		};

		/* ---- E1: move draws of the outputs, per-class counts; with room for
		 * a word per output and offsets that fit 11 bits (at most 2048
		 * outputs), each output's cell in its destination tile (bits 0-12),
		 * direction (13-15; DIR_DROPPED for an output counted nowhere),
		 * class (16-20) and offset in its class's group (21-31) are kept for
		 * E2, else only its direction. The room: the cell counters' words
		 * (T, enough when 2 act_cap <= T); in split tiles the counters, the
		 * grass words after them (T / 2 words, dead after the actions) and
		 * the permutation array past the output map, per tile as its
		 * outputs need ---- */
		bool bad = false;
		constexpr uint32_t DEST_A = CPT * NT + CPT * NT / 2;
		const uint32_t dest_b0 = (total + 1) / 2;    /* words of the output map */
		const bool cache = in_smem && (split
			? total <= 2048u && total <= DEST_A + (w.act_cap - dest_b0)
			: 2u * w.act_cap <= 2048u);
		uint32_t *DEST = scnt;
		auto dest = [&](uint32_t o) -> uint32_t & {
			if (!split || o < DEST_A) return DEST[o];
			return PERM[dest_b0 + (o - DEST_A)];
		};
		for (uint32_t o = tid; o < total; o += NT) {
			uint32_t j, nb, en, rank;
			output(o, j, nb, en, rank);
			const uint32_t lc = LK[j] & 0xffffu;
			uint32_t code, cls, klo = lc;
			if (!live_move) {
				code = DIR_PARKED;
				cls = CLS_GRAVE;
			} else if (((en - 1) & run.emask) == 0) {
				code = DIR_DEAD;
				cls = CLS_GRAVE;
			} else {
				const u4 r = rng(seed_lo, seed_hi, lt0 + lc, tmove, STREAM_MOVE, rank);
				code = draw(r.x, 5);
				const uint32_t dg = run.cbase + move_dir(run, lt0 + lc, code);
				const uint32_t dt = dg >> w.log_tile;
				klo = dg & lcmask;
				cls = dt == tile ? CLS_OWN : class_insert(s_tbl, dt);
			}
			if (cls == CLS_NONE || rank > REC_RANK_MAX) {
				bad = true;
				cls = NCLS;                      /* counted nowhere */
			}
			const uint32_t off = warp_agg_add(s_ccnt, cls);
			if (cache)
				dest(o) = cls == NCLS ? DIR_DROPPED << REC_DIR_SHIFT
					: klo | (code << REC_DIR_SHIFT) | (cls << 16) | (off << 21);
			else DIR[o] = (uint8_t) code;
		}
		if (bad) atomicOr(&w.ctr->err, ERRF_OVERFLOW);
		__syncthreads();

		/* ---- the tile's groups: one per class, laid out in class order
		 * from its slots ---- */
		uint32_t my_c = 0, my_start = 0;
		if (tid < 32) {
			my_c = s_ccnt[lane];
			uint32_t x = my_c;
#pragma unroll
			for (int o = 1; o < 32; o <<= 1) {
				const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
				if (lane >= (uint32_t) o) x += y;
			}
			const bool fail = (uint64_t) gb + total > 3ull * w.cap;
			if (lane == 0) {
				s_fail = fail;
				if (fail) atomicOr(&w.ctr->err, ERRF_OVERFLOW);
			}
			my_start = gb + x - my_c;
			s_cpos[lane] = my_start;
		}
		__syncthreads();

		if (!s_fail) {
			/* the groups are posted to their destination tiles' inboxes by
			 * warp 0 while the records are written */
			uint32_t slot = IBX;
			size_t ib = 0;
			if (tid < 32 && my_c) {
				const uint32_t dt = lane < CLS_FOREIGN ? s_tbl[lane] : tile;
				ib = (size_t) pout * w.n_tiles + dt;
				slot = atomicAdd(&w.inbox_n[ib], 1u);
			}
			/* ---- E2: records into the groups ---- */
			uint32_t *kGo = pout ? w.kG1 : w.kG0;
			uint32_t *vGo = pout ? w.vG1 : w.vG0;
			for (uint32_t o = tid; o < total; o += NT) {
				uint32_t j, nb, en, rank;
				output(o, j, nb, en, rank);
				const uint32_t lc = LK[j] & 0xffffu;
				const uint32_t tb = LV[j] & TYPE_BIT;
				uint32_t key, val, cls;
				if (cache) {
					const uint32_t d = dest(o);
					const uint32_t code = (d >> REC_DIR_SHIFT) & 7u;
					cls = (d >> 16) & 31u;
					key = (d & 0xffffu) | (rank << REC_RANK_SHIFT);
					val = code >= DIR_PARKED ? (tb | en) : (tb | ((en - 1) & run.emask));
					const uint32_t pos = s_cpos[cls] + (d >> 21);
					if (code != DIR_DROPPED) {
						kGo[pos] = key;
						vGo[pos] = val;
					}
					continue;
				}
				const uint32_t code = DIR[o];
				if (code >= DIR_PARKED) {
					cls = CLS_GRAVE;
					key = lc | (code << REC_DIR_SHIFT) | (rank << REC_RANK_SHIFT);
					val = tb | en;
				} else {
					const uint32_t dg = run.cbase + move_dir(run, lt0 + lc, code);
					const uint32_t dt = dg >> w.log_tile;
					cls = dt == tile ? CLS_OWN : class_find(s_tbl, dt);
					key = (dg & lcmask) | (code << REC_DIR_SHIFT) | (rank << REC_RANK_SHIFT);
					val = tb | ((en - 1) & run.emask);
				}
				if (cls == CLS_NONE || rank > REC_RANK_MAX) cls = NCLS;
				const uint32_t pos = warp_agg_add(s_cpos, cls);
				if (cls != NCLS) {
					kGo[pos] = key;
					vGo[pos] = val;
				}
			}
			if (tid < 32 && my_c) {
				if (slot < IBX)
					w.inbox[ib * IBX + slot] = make_uint2(my_start,
						my_c | (lane == CLS_GRAVE ? GROUP_GRAVE : 0u));
				else
					atomicOr(&w.ctr->err, ERRF_OVERFLOW);
			}
		}

		/* ---- per-tile partial stats (ACT); the tile's eating events go to the
		 * run's regrowth histogram slot of iteration t + restart ---- */
		if (ACT) {
			const uint32_t wid = tid >> 5;
			const uint32_t sw = warp_sum(sheep | (wolves << 16));
			const uint32_t ew = warp_sum(eats);
			/* energy sums: one 32-bit warp reduction each while every
			 * lane's sum is below 2^26 (32 of them stay below 2^31) */
			uint64_t se, we;
			if (__all_sync(0xffffffffu, ((sen | wen) >> 26) == 0)) {
				se = __reduce_add_sync(0xffffffffu, (uint32_t) sen);
				we = __reduce_add_sync(0xffffffffu, (uint32_t) wen);
			} else {
				se = warp_sum(sen);
				we = warp_sum(wen);
			}
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
				for (uint32_t q = 0; q < NT / 32; q++) sum += red[tid][q];
				if (tid == 2) {
					if (sum)
						atomicAdd(&w.fring[run.fbase + (t + run.restart) % (run.restart + 1)],
							(uint32_t) sum);
					w.part[(size_t) tile * 8 + 2] = 0;
					w.part[(size_t) tile * 8 + 5] = 0;
				} else {
					w.part[(size_t) tile * 8 + tid] = sum;
				}
			}
		}
	};
	if (in_smem) {
		if (2u * w.act_cap <= (uint32_t) (CPT * NT))
			phases(std::true_type{}, std::false_type{}, sk, sv, sperm, sp, sd);
		else
			phases(std::true_type{}, std::true_type{}, sk, sv, sperm, sp, sd);
	} else {
		const uint32_t xb = s_xbase;
		phases(std::false_type{}, std::false_type{}, w.scratch_prio + xb,
			w.scratch_kid + xb, w.scratch_perm + 3ull * xb, w.scratch_key + xb,
			w.scratch_val + xb);
	}
}

/* The fused act: one CTA per tile below the world's high-water mark (the
 * host sizes the grid from it and moves it when runs are admitted or
 * retired), so a serving world's free tile space costs nothing. */
template <int CPT, int NT>
__global__ void __launch_bounds__(NT, CTAS_PER_SM(NT)) k_step_act(WorldDev w)
{
	extern __shared__ __align__(16) uint32_t sm[];
	if (blockIdx.x >= min(w.ctr->tile_hi, w.n_tiles)) return;
	step_tile<CPT, NT, true>(w, blockIdx.x, 0, sm);
}

/* The first move of a freshly initialised run: one CTA per tile of
 * [tile0, tile0 + gridDim.x). */
template <int CPT, int NT>
__global__ void __launch_bounds__(NT, CTAS_PER_SM(NT)) k_step_first(WorldDev w,
	uint32_t tile0, uint32_t out_base)
{
	extern __shared__ __align__(16) uint32_t sm[];
	step_tile<CPT, NT, false>(w, tile0 + blockIdx.x, out_base, sm);
}

template <int CPT, int NT, bool ACT>
void launch_one(const WorldDev &w, uint32_t grid, size_t smem, uint32_t first,
	uint32_t out_base, cudaStream_t s)
{
	if (ACT) k_step_act<CPT, NT><<<grid, NT, smem, s>>>(w);
	else k_step_first<CPT, NT><<<grid, NT, smem, s>>>(w, first, out_base);
}

/* Thread count of a world's tile CTAs (see NT_SPARSE / NT_DENSE). */
inline int step_threads_for(uint32_t T, uint32_t act_cap)
{
	return 2u * act_cap > T && T >= 1024 ? NT_DENSE : NT_SPARSE;
}

inline int step_threads(const WorldDev &w)
{
	return step_threads_for(1u << w.log_tile, w.act_cap);
}

/* Dynamic shared memory of a tile CTA: five agent arrays of act_cap words,
 * then the cell counters (a word a cell) and the grass (two bytes a cell). */
inline size_t step_smem(uint32_t T, uint32_t act_cap)
{
	return (size_t) act_cap * 5 * sizeof(uint32_t)
		+ (size_t) T * (sizeof(uint32_t) + sizeof(uint16_t));
}

template <bool ACT>
cudaError_t launch_step(const WorldDev &w, const LaunchCfg &lc, uint32_t first,
	uint32_t count, uint32_t out_base, cudaStream_t s)
{
	const uint32_t T = 1u << w.log_tile;
	const size_t smem = step_smem(T, w.act_cap);
	const uint32_t grid = ACT ? (uint32_t) std::max(1, lc.act_tiles) : count;
	if (step_threads(w) == NT_DENSE) {
		switch (T / NT_DENSE) {
		case 4: launch_one<4, NT_DENSE, ACT>(w, grid, smem, first, out_base, s); break;
		case 8: launch_one<8, NT_DENSE, ACT>(w, grid, smem, first, out_base, s); break;
		case 16: launch_one<16, NT_DENSE, ACT>(w, grid, smem, first, out_base, s); break;
		default: launch_one<32, NT_DENSE, ACT>(w, grid, smem, first, out_base, s); break;
		}
	} else {
		switch (T / NT_SPARSE) {
		case 4: launch_one<4, NT_SPARSE, ACT>(w, grid, smem, first, out_base, s); break;
		case 8: launch_one<8, NT_SPARSE, ACT>(w, grid, smem, first, out_base, s); break;
		case 16: launch_one<16, NT_SPARSE, ACT>(w, grid, smem, first, out_base, s); break;
		case 32: launch_one<32, NT_SPARSE, ACT>(w, grid, smem, first, out_base, s); break;
		default: launch_one<64, NT_SPARSE, ACT>(w, grid, smem, first, out_base, s); break;
		}
	}
	return cudaGetLastError();
}

template <int CPT, int NT>
cudaError_t set_step_limit(size_t bytes)
{
	cudaError_t e = cudaFuncSetAttribute(k_step_act<CPT, NT>,
		cudaFuncAttributeMaxDynamicSharedMemorySize, (int) bytes);
	if (e != cudaSuccess) return e;
	return cudaFuncSetAttribute(k_step_first<CPT, NT>,
		cudaFuncAttributeMaxDynamicSharedMemorySize, (int) bytes);
}

} /* namespace */

cudaError_t enqueue_iteration_fused(const WorldDev &w, const LaunchCfg &lc,
	cudaStream_t s, const cudaEvent_t *marks)
{
	/* marks (optional, 3 events): before the act, after it, after the
	 * finish */
	if (marks) cudaEventRecord(marks[0], s);
	cudaError_t e = launch_step<true>(w, lc, 0, w.n_tiles, 0, s);
	if (e != cudaSuccess) return e;
	if (marks) cudaEventRecord(marks[1], s);
	e = launch_finish_fused(w, lc, s);
	if (marks) cudaEventRecord(marks[2], s);
	return e;
}

cudaError_t enqueue_move_groups(const WorldDev &w, const LaunchCfg &lc,
	uint32_t first, uint32_t count, uint32_t out_base, cudaStream_t s)
{
	if (count == 0) return cudaSuccess;
	return launch_step<false>(w, lc, first, count, out_base, s);
}

int step_ctas_per_sm(uint32_t log_tile, uint32_t act_cap)
{
	const uint32_t T = 1u << log_tile;
	const size_t smem = step_smem(T, act_cap);
	int n = 0;
	cudaError_t e;
	if (step_threads_for(T, act_cap) == NT_DENSE) {
		switch (T / NT_DENSE) {
		case 4: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_step_act<4, NT_DENSE>, NT_DENSE, smem); break;
		case 8: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_step_act<8, NT_DENSE>, NT_DENSE, smem); break;
		case 16: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_step_act<16, NT_DENSE>, NT_DENSE, smem); break;
		default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_step_act<32, NT_DENSE>, NT_DENSE, smem); break;
		}
	} else {
		switch (T / NT_SPARSE) {
		case 4: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_step_act<4, NT_SPARSE>, NT_SPARSE, smem); break;
		case 8: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_step_act<8, NT_SPARSE>, NT_SPARSE, smem); break;
		case 16: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_step_act<16, NT_SPARSE>, NT_SPARSE, smem); break;
		case 32: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_step_act<32, NT_SPARSE>, NT_SPARSE, smem); break;
		default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_step_act<64, NT_SPARSE>, NT_SPARSE, smem); break;
		}
	}
	if (e != cudaSuccess) {
		cudaGetLastError();
		return 0;
	}
	return n;
}

uint32_t grow_act_cap(uint32_t log_tile, uint32_t act_cap)
{
	const uint32_t T = 1u << log_tile;
	if (set_step_smem_limits(step_smem(T, 2 * T)) != cudaSuccess) {
		cudaGetLastError();
		return act_cap;
	}
	/* the record cache of the move phase needs 2 act_cap <= T and
	 * 2 act_cap <= 2048 (pp_fused.cu E1) */
	auto cache_ok = [&](uint32_t a) { return 2u * a <= T && 2u * a <= 2048u; };
	const int occ = step_ctas_per_sm(log_tile, act_cap);
	const int nt = step_threads_for(T, act_cap);
	const bool cached = cache_ok(act_cap);
	if (occ <= 0) return act_cap;
	for (uint32_t a = act_cap + 32; a <= 2 * T; a += 32) {
		if (step_threads_for(T, a) != nt || (cached && !cache_ok(a))
			|| step_ctas_per_sm(log_tile, a) < occ)
			break;
		act_cap = a;
	}
	return act_cap;
}

cudaError_t set_step_smem_limits(size_t bytes)
{
	cudaError_t e = set_step_limit<4, NT_SPARSE>(bytes);
	if (e == cudaSuccess) e = set_step_limit<8, NT_SPARSE>(bytes);
	if (e == cudaSuccess) e = set_step_limit<16, NT_SPARSE>(bytes);
	if (e == cudaSuccess) e = set_step_limit<32, NT_SPARSE>(bytes);
	if (e == cudaSuccess) e = set_step_limit<64, NT_SPARSE>(bytes);
	if (e == cudaSuccess) e = set_step_limit<4, NT_DENSE>(bytes);
	if (e == cudaSuccess) e = set_step_limit<8, NT_DENSE>(bytes);
	if (e == cudaSuccess) e = set_step_limit<16, NT_DENSE>(bytes);
	if (e == cudaSuccess) e = set_step_limit<32, NT_DENSE>(bytes);
	return e;
}

} /* namespace pp */
