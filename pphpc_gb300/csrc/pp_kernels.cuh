/*
 * pp_kernels.cuh -- launch wrappers of the simulation kernels (defined in
 * pp_kernels.cu and pp_radix.cu).
 */
#pragma once

#include "pp_device.cuh"
#include "../../include/pphpc.h"

namespace pp {

/* Everything one world iteration touches. Sort pipeline: the state between
 * iterations is the region buffer R: tile t's agents (its cells' lists,
 * cell-sorted) at [rstart[t], rstart[t] + rcnt[t]), with dense base
 * dbase[t]. The move reads the regions into the dense array B, the radix
 * passes ping-pong B <-> C, the act reads the sorted array and writes each
 * tile's region at twice its sorted offset. A (cap slots) is a dense copy
 * for read-back. Both pipelines create agents into B. Arrays a pipeline
 * does not use are not allocated (null). */
struct WorldDev {
	uint16_t *grass;          /* regrowth iteration per cell (see pp_device.cuh) */
	uint32_t *fring;          /* per-run histograms of pending regrowth iterations */
	uint32_t *kA, *vA, *kB, *vB, *kC, *vC;
	uint32_t *kR, *vR;        /* region buffer, 3 * cap slots              */
	uint32_t *rstart, *rcnt;  /* n_tiles                                   */
	uint32_t *dbase;          /* n_tiles + 1                               */
	uint32_t *tile_off;       /* n_tiles + 1                               */
	uint16_t *tile_run;       /* n_tiles                                   */
	RunDev *runs;             /* nruns_cap                                 */
	uint64_t *lb_sort;        /* sort look-back words [max sort tiles][radix] */
	uint64_t *lb_fin;         /* finish look-back words [n_tiles + 1]      */
	WorldCounters *ctr;
	uint32_t *hist;           /* [8][256] digit counts of the moved keys   */
	PPStatistics *ring;       /* [ring_rows][nruns_cap]                    */
	uint32_t *scratch_key, *scratch_val, *scratch_prio, *scratch_kid,
		*scratch_perm;        /* [cap], act fallback for crowded tiles     */
	uint64_t *part;           /* [n_tiles][8] per-tile partial stats       */
	uint32_t cap, n_tiles, log_tile, nruns_cap, ring_rows;
	uint32_t key_bits, digit_bits, passes;
	uint32_t sort_shift;      /* the sort orders key bits [sort_shift, key_bits) */
	uint32_t act_cap;         /* agents per tile held in shared memory     */
	uint32_t dead_key;        /* = n_tiles << log_tile                      */
	/* fused pipeline: the state between iterations is, per parity, a group
	 * buffer of moved agents (records, see pp_device.cuh) and per tile an
	 * inbox listing the groups destined to it */
	uint32_t *kG0, *vG0, *kG1, *vG1;   /* group buffers, 3 * cap slots each: the
	                           act of tile t writes at 2 * dbase[t] (dbase =
	                           dense base of its next-act inputs), admitted
	                           runs' first moves from 2 * cap on */
	uint2 *inbox;             /* [2][n_tiles][IBX]                          */
	uint32_t *inbox_n;        /* [2][n_tiles]                               */
	uint4 *bucket;            /* [cap] initial agents bucketed by tile: cell,
	                           type | energy, creation index (fused only)  */
	uint32_t *bscan;          /* [n_tiles / 4096 + 2] bucket scan partials  */
	FocalDev *focal;          /* [nruns_cap] running focal measures         */
	uint32_t fused;
};

struct LaunchCfg {
	int sms;
	int move_blocks, sort_blocks, offs_blocks, finish_blocks;
	int act_tiles;            /* fused act grid: tiles below the high-water mark */
	int cpt;                  /* cells per act thread (4, 8, 16 or 32)      */
};

/* Sort tile geometry. */
constexpr int SORT_THREADS = 256;
constexpr int SORT_IPT = 16;
constexpr int SORT_TILE = SORT_THREADS * SORT_IPT;
constexpr int ACT_THREADS = 256;

/* One iteration: move, radix passes, tile offsets, act, finish. Returns a
 * CUDA error code (cudaSuccess = 0). */
cudaError_t enqueue_iteration(const WorldDev &w, const LaunchCfg &lc,
	cudaStream_t s, const cudaEvent_t *marks = nullptr);

/* One fused iteration: act+move (gather by destination tile), finish. */
cudaError_t enqueue_iteration_fused(const WorldDev &w, const LaunchCfg &lc,
	cudaStream_t s, const cudaEvent_t *marks = nullptr);

/* Fused pipeline: the first move of the agents of tiles [first, first +
 * count), bucketed by tile in w.bucket (tile offsets in w.tile_off), into
 * the group buffer the next act reads. */
cudaError_t enqueue_move_groups(const WorldDev &w, const LaunchCfg &lc,
	uint32_t first, uint32_t count, uint32_t out_base, cudaStream_t s);

/* Fused pipeline: the n agents in kB/vB (creation order) bucketed by tile
 * into w.bucket with their creation indices; tile offsets of tiles [first,
 * first + count] in w.tile_off (tile_off[first + count] = n), which must be
 * zero on entry. */
cudaError_t enqueue_bucket_agents(const WorldDev &w, uint32_t n,
	uint32_t first, uint32_t count, cudaStream_t s);

/* Fused pipeline: dense bases of the next act's per-tile inputs (after a
 * first move outside an iteration). */
cudaError_t enqueue_fused_bases(const WorldDev &w, const LaunchCfg &lc,
	cudaStream_t s);

cudaError_t set_step_smem_limits(size_t bytes);

/* Fused act CTAs per SM for tiles of 2^log_tile cells with act_cap agents
 * in shared memory (0 if the query fails). */
int step_ctas_per_sm(uint32_t log_tile, uint32_t act_cap);

/* The largest act_cap (in steps of 32) above the given one that keeps its
 * CTAs per SM, its CTA size and its move-phase record cache: more agents
 * held in shared memory at no cost in occupancy. */
uint32_t grow_act_cap(uint32_t log_tile, uint32_t act_cap);

/* Bounded look-back self-test over n chunks (chunk `stall` never
 * publishes; `limit` polls per wait). */
cudaError_t launch_lookback_selftest(uint64_t *lb, uint32_t *ticket, uint32_t *err,
	uint32_t *prefix, uint32_t n, uint32_t stall, uint32_t limit, cudaStream_t s);

/* Focal measures of run r restarted from its stats row `row` (its
 * iteration t0). */
cudaError_t enqueue_focal_init(const WorldDev &w, uint32_t r, uint32_t row,
	uint32_t t0, cudaStream_t s);

/* Initialisation of run r: grass of its tiles; its initial agents in
 * creation order into k/v[base ..) (bucketed or sorted by cell
 * afterwards). Each adds its part of the run's stats (live cells and
 * countdown sum; agent counts and energy sums) to ring row `row`. */
cudaError_t enqueue_init_grass(const WorldDev &w, const RunDev &run,
	uint32_t r, uint32_t row, cudaStream_t s);
cudaError_t enqueue_init_agents(const WorldDev &w, const RunDev &run,
	uint32_t r, uint32_t row, uint32_t *k, uint32_t *v, uint32_t base,
	uint32_t init_sheep, uint32_t init_wolves, cudaStream_t s);
/* Regions of tiles [first, first + count) for a cell-sorted array of
 * ctr->aux_n agents at region-buffer offset `base`, then the dense bases
 * of all regions. */
cudaError_t enqueue_regions_from_sorted(const WorldDev &w, const LaunchCfg &lc,
	const uint32_t *sorted_keys, uint32_t first, uint32_t count,
	uint32_t base, cudaStream_t s);
/* Dense copy of all regions into ko/vo (dbase order). */
cudaError_t enqueue_compact(const WorldDev &w, const LaunchCfg &lc,
	uint32_t *ko, uint32_t *vo, cudaStream_t s);
/* Move the regrowth iteration of alive cells to their run's current
 * iteration (keeps the 16-bit representation from wrapping). */
cudaError_t enqueue_grass_rebase(const WorldDev &w, const LaunchCfg &lc,
	cudaStream_t s);
/* After a standalone sort that used the world's counters: new look-back
 * epochs, fresh tickets, zero histograms. */
cudaError_t enqueue_after_sort(WorldCounters *ctr, uint32_t *hist,
	cudaStream_t s);

/* Standalone kernels for kernel-level checks. */
cudaError_t launch_move_only(const uint32_t *kin, const uint32_t *vin,
	uint32_t *kout, uint32_t *vout, uint32_t n, const RunDev *run_dev,
	uint32_t iter, uint32_t dead_key, cudaStream_t s);

cudaError_t launch_offsets(const uint32_t *keys, const uint32_t *n_dev,
	uint32_t log_tile, uint32_t n_buckets, uint32_t *off, int blocks,
	cudaStream_t s);

cudaError_t launch_philox_fill(uint32_t c0, uint32_t c1, uint32_t c2,
	uint32_t c3, uint32_t k0, uint32_t k1, uint32_t n, uint32_t *out,
	cudaStream_t s);

/* Radix sort primitives (pp_radix.cu). */
cudaError_t launch_radix_hist(const uint32_t *keys, const uint32_t *n_dev,
	uint32_t *hist, uint32_t digit_bits, uint32_t passes, int blocks,
	cudaStream_t s);

cudaError_t launch_radix_pass(const uint32_t *kin, const uint32_t *vin,
	uint32_t *kout, uint32_t *vout, const uint32_t *hist_pass,
	uint64_t *lb, WorldCounters *ctr, const uint32_t *n_dev, uint32_t pass,
	uint32_t shift, uint32_t digit_bits, int blocks, cudaStream_t s);

} /* namespace pp */
