/*
 * pp_world.cu -- world management and the C ABI of single simulations,
 * batched runs and kernel-level entry points.
 *
 * The reference's host loop (opencl/pp/pp_gpu.c:573-987) blocks on the
 * host every iteration to read the stats and size the next launches
 * (pp_gpu.c:840-852). Here every kernel reads its sizes from device
 * counters, so an iteration is a fixed launch sequence; `graph_iters`
 * iterations are captured once into a CUDA graph and replayed, and the
 * host synchronises only every `ring_rows - 1` iterations to copy the
 * stats ring out and check the overflow/timeout flags.
 */
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <new>

#include "pp_world.cuh"
#include "pp_act.cuh"

namespace pp {

cudaError_t set_act_smem_limits(size_t bytes);
int occupancy_act(int cpt, size_t smem);
int occupancy_sort(int dbits);

int cuda_status(cudaError_t e)
{
	if (e == cudaSuccess) return PP_SUCCESS;
	if (e == cudaErrorMemoryAllocation) return PP_OUT_OF_RESOURCES;
	return PP_ERR_CUDA;
}

#define PP_CK(call) do { cudaError_t e_ = (call); \
	if (e_ != cudaSuccess) return cuda_status(e_); } while (0)

static uint32_t ceil_div(uint64_t a, uint64_t b) { return (uint32_t) ((a + b - 1) / b); }

static uint32_t pow2_ceil(uint32_t v)
{
	uint32_t p = 1;
	while (p < v) p <<= 1;
	return p;
}

void choose_geometry(uint32_t total_cells, uint32_t cap, WorldConfig &cfg)
{
	if (cfg.tile_cells == 0) {
		/* Dense worlds (many agents per cell) take smaller tiles so a
		 * tile's agents fit in shared memory (the fused act: 512-cell
		 * tiles of 128 threads); the fused act is latency bound per tile
		 * and prefers more, smaller tiles in flight (nine 128-thread CTAs
		 * per SM) than the sort pipeline's act. */
		double dens = total_cells ? (double) cap / total_cells : 1.0;
		if (dens > 1.0) cfg.tile_cells = cfg.fused ? 512 : 1024;
		else cfg.tile_cells = cfg.fused ? 2048 : 4096;
	}
}

World::~World() { free_all(); }

void World::free_all()
{
	if (device_ >= 0 && !allocs_.empty()) cudaSetDevice(device_);
	drop_graph();
	/* the buffers go back to the process cache only once no work of this
	 * world can still touch them */
	if (s_) cudaStreamSynchronize(s_);
	for (auto &a : allocs_) cached_free(device_, a.first, a.second);
	allocs_.clear();
	if (s_) cudaStreamDestroy(s_);
	s_ = nullptr;
}

int World::alloc(size_t bytes, void **p)
{
	if (bytes == 0) bytes = 16;
	size_t got = 0;
	cudaError_t e = cached_malloc(device_, bytes, p, &got);
	if (e != cudaSuccess) {
		cudaGetLastError();
		return e == cudaErrorMemoryAllocation ? PP_OUT_OF_RESOURCES : PP_ERR_CUDA;
	}
	allocs_.emplace_back(*p, got);
	bytes_ += bytes;
	return PP_SUCCESS;
}

static RunDev make_run(const RunSpec &s, uint32_t first_tile,
	uint32_t n_tiles, uint32_t log_tile, uint32_t start_giter, uint32_t fbase)
{
	RunDev r{};
	r.gx = s.p.grid_x;
	r.gy = s.p.grid_y;
	r.ncells = s.p.grid_x * s.p.grid_y;
	r.cbase = first_tile << log_tile;
	r.first_tile = first_tile;
	r.n_tiles = n_tiles;
	r.sheep_gain = s.p.sheep_gain_from_food;
	r.sheep_thr = s.p.sheep_reproduce_threshold;
	r.sheep_prob = s.p.sheep_reproduce_prob;
	r.wolves_gain = s.p.wolves_gain_from_food;
	r.wolves_thr = s.p.wolves_reproduce_threshold;
	r.wolves_prob = s.p.wolves_reproduce_prob;
	r.restart = s.p.grass_restart;
	r.seed_lo = (uint32_t) s.seed;
	r.seed_hi = (uint32_t) (s.seed >> 32);
	r.iters = s.iters;
	r.start_giter = start_giter;
	r.active = 1;
	r.fbase = fbase;
	r.ss_from = s.ss_from;
	r.emask = energy_mask_of(s.energy_bits);
	r.gxdiv = fastdiv_make(s.p.grid_x);
	return r;
}

int agent_energy_bits(uint32_t agent_size, const PPParameters &p, uint32_t *bits)
{
	switch (agent_size) {
	case 0: *bits = 30; return PP_SUCCESS;
	case 64: *bits = 16; return PP_SUCCESS;
	case 32:
		if (p.grid_x > 1024 || p.grid_y > 1024) return PP_INVALID_ARGS;
		*bits = 11;
		return PP_SUCCESS;
	default: return PP_INVALID_ARGS;
	}
}

int World::create(const std::vector<RunSpec> &runs, const WorldConfig &cfg_in)
{
	pp::NvtxRange nvtx_range("world create");
	WorldConfig cfg = cfg_in;
	device_ = cfg.device;
	PP_CK(cudaSetDevice(device_));
	PP_CK(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking));
	int sms = 0;
	PP_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));

	uint64_t total_cells = 0, n0 = 0;
	for (const RunSpec &r : runs) {
		total_cells += (uint64_t) r.p.grid_x * r.p.grid_y;
		n0 += r.agents();
	}
	if (cfg.cap == 0) cfg.cap = (uint32_t) std::min<uint64_t>(
		std::max<uint64_t>(4 * n0, 1024), 0x7fffffffu);
	if (n0 > cfg.cap) return PP_OUT_OF_RESOURCES;
	choose_geometry((uint32_t) std::min<uint64_t>(total_cells, 0xffffffffu),
		cfg.cap, cfg);
	uint32_t T = cfg.tile_cells;
	if (T != 1024 && T != 2048 && T != 4096 && T != 8192
		&& !(T == 512 && cfg.fused)) return PP_INVALID_ARGS;
	uint32_t log_tile = 0;
	while ((1u << log_tile) < T) log_tile++;

	uint64_t tiles = 0;
	std::vector<uint32_t> first(runs.size()), ntl(runs.size());
	for (size_t r = 0; r < runs.size(); r++) {
		uint64_t c = (uint64_t) runs[r].p.grid_x * runs[r].p.grid_y;
		first[r] = (uint32_t) tiles;
		ntl[r] = ceil_div(c, T);
		tiles += ntl[r];
	}
	used_tiles_ = (uint32_t) tiles;
	tiles += cfg.extra_tiles;
	if (tiles == 0) tiles = 1;
	if ((tiles << log_tile) >= 0x80000000ull) return PP_INVALID_ARGS;

	uint32_t nruns_cap = std::max<uint32_t>(cfg.nruns_cap, (uint32_t) runs.size()) + 1;
	null_slot_ = nruns_cap - 1;
	if (nruns_cap > 65535) return PP_INVALID_ARGS;

	w_.cap = cfg.cap;
	w_.fused = cfg.fused ? 1u : 0u;
	w_.n_tiles = (uint32_t) tiles;
	w_.log_tile = log_tile;
	w_.nruns_cap = nruns_cap;
	w_.ring_rows = std::max<uint32_t>(cfg.ring_rows, 16);
	w_.dead_key = (uint32_t) (tiles << log_tile);
	uint32_t kb = 32 - __builtin_clz(w_.dead_key);
	w_.key_bits = kb;
	/* The act groups a tile's agents by cell itself, so the sort orders
	 * only the tile bits of the cell key. */
	w_.sort_shift = log_tile;
	const uint32_t sb = kb > log_tile ? kb - log_tile : 1;
	uint32_t d = cfg.digit_bits;
	if (d == 0) {
		uint32_t passes = (sb + 7) / 8;
		d = (sb + passes - 1) / passes;
	}
	if (d < 5) d = 5;
	if (d > 8) return PP_INVALID_ARGS;
	w_.digit_bits = d;
	w_.passes = (sb + d - 1) / d;
	if (w_.passes > 8) return PP_INVALID_ARGS;

	uint32_t act_cap = cfg.act_cap;
	if (act_cap == 0) {
		double dens = total_cells ? (double) cfg.cap / (double) total_cells : 2.0;
		if (dens > 2.0) dens = 2.0;
		act_cap = pow2_ceil((uint32_t) (T * dens * 0.75) + 1);
		act_cap = std::min<uint32_t>(std::max<uint32_t>(act_cap, 256), 4096);
	}
	/* the fused act keeps a byte per output (at most 2 act_cap) in the
	 * tile's 4 T bytes of cell counters */
	act_cap = std::min<uint32_t>(act_cap, 2 * T);
	/* fused pipeline: the shared memory the chosen act_cap leaves unused at
	 * its CTAs per SM holds more agents (12800^2, 2048-cell tiles: 512 ->
	 * 576, so fewer tiles at the population peak take the crowded path) */
	if (cfg.fused && cfg.act_cap == 0) act_cap = grow_act_cap(log_tile, act_cap);
	w_.act_cap = act_cap;

	const size_t cap = cfg.cap;
	int rc;
#define PP_AL(ptr, bytes) do { void *p_; rc = alloc((bytes), &p_); \
	if (rc) return rc; (ptr) = (decltype(ptr)) p_; } while (0)
	PP_AL(w_.grass, (size_t) w_.dead_key * sizeof(uint16_t));
	PP_AL(w_.kB, cap * 4); PP_AL(w_.vB, cap * 4);
	if (w_.fused) {
		PP_AL(w_.bucket, cap * 16);
		PP_AL(w_.bscan, ((size_t) tiles / 4096 + 2) * 4);
		PP_AL(w_.kG0, 3 * cap * 4); PP_AL(w_.vG0, 3 * cap * 4);
		PP_AL(w_.kG1, 3 * cap * 4); PP_AL(w_.vG1, 3 * cap * 4);
		PP_AL(w_.inbox, (size_t) 2 * tiles * IBX * sizeof(uint2));
		PP_AL(w_.inbox_n, (size_t) 2 * tiles * 4);
	} else {
		PP_AL(w_.kA, cap * 4); PP_AL(w_.vA, cap * 4);
		PP_AL(w_.kC, cap * 4); PP_AL(w_.vC, cap * 4);
		PP_AL(w_.kR, 3 * cap * 4); PP_AL(w_.vR, 3 * cap * 4);
	}
	PP_AL(w_.scratch_key, cap * 4); PP_AL(w_.scratch_val, cap * 4);
	PP_AL(w_.scratch_prio, cap * 4); PP_AL(w_.scratch_kid, cap * 4);
	PP_AL(w_.scratch_perm, (w_.fused ? 3 : 1) * cap * 4);
	PP_AL(w_.rstart, (size_t) tiles * 4);
	PP_AL(w_.rcnt, (size_t) tiles * 4);
	PP_AL(w_.dbase, ((size_t) tiles + 1) * 4);
	PP_AL(w_.tile_off, ((size_t) tiles + 1) * 4);
	PP_AL(w_.tile_run, (size_t) tiles * 2);
	PP_AL(w_.runs, (size_t) nruns_cap * sizeof(RunDev));
	PP_AL(w_.part, (size_t) tiles * 8 * sizeof(uint64_t));
	PP_AL(w_.focal, (size_t) nruns_cap * sizeof(FocalDev));
	size_t sort_tiles = ceil_div(cap, SORT_TILE) + 1;
	PP_AL(w_.lb_sort, sort_tiles * 256 * sizeof(uint64_t));
	PP_AL(w_.lb_fin, ((size_t) tiles + 1) * sizeof(uint64_t));
	PP_AL(w_.ctr, sizeof(WorldCounters));
	PP_AL(w_.hist, 8 * 256 * 4);
	PP_AL(w_.ring, (size_t) w_.ring_rows * nruns_cap * sizeof(PPStatistics));
	/* regrowth histograms: restart + 1 slots per initial run, and room for
	 * any restart in every slot left for later admissions */
	std::vector<uint32_t> fbase_h(runs.size());
	uint64_t fsz = 0;
	for (size_t r = 0; r < runs.size(); r++) {
		fbase_h[r] = (uint32_t) fsz;
		fsz += runs[r].p.grass_restart + 1;
	}
	fslot_base_ = (uint32_t) fsz;
	fsz += (uint64_t) (nruns_cap - 1 - runs.size()) * FSLOT;
	PP_AL(w_.fring, std::max<uint64_t>(fsz, 1) * 4);
#undef PP_AL
	PP_CK(cudaMemsetAsync(w_.lb_sort, 0, sort_tiles * 256 * sizeof(uint64_t), s_));
	PP_CK(cudaMemsetAsync(w_.lb_fin, 0, ((size_t) tiles + 1) * sizeof(uint64_t), s_));
	PP_CK(cudaMemsetAsync(w_.rcnt, 0, (size_t) tiles * 4, s_));
	PP_CK(cudaMemsetAsync(w_.rstart, 0, (size_t) tiles * 4, s_));
	PP_CK(cudaMemsetAsync(w_.hist, 0, 8 * 256 * 4, s_));
	PP_CK(cudaMemsetAsync(w_.ring, 0, (size_t) w_.ring_rows * nruns_cap * sizeof(PPStatistics), s_));
	PP_CK(cudaMemsetAsync(w_.part, 0, (size_t) tiles * 8 * sizeof(uint64_t), s_));
	PP_CK(cudaMemsetAsync(w_.fring, 0, std::max<uint64_t>(fsz, 1) * 4, s_));
	if (w_.fused) PP_CK(cudaMemsetAsync(w_.inbox_n, 0, (size_t) 2 * tiles * 4, s_));

	/* Run table and tile map. */
	runs_h_.assign(nruns_cap, RunDev{});
	reserve_of_.assign(nruns_cap, 0);
	tile_run_h_.assign(tiles, (uint16_t) null_slot_);
	std::vector<uint32_t> base_h(nruns_cap, 0);
	uint32_t base = 0;
	for (size_t r = 0; r < runs.size(); r++) {
		/* a resumed run's iteration t is the world's iteration plus its
		 * start iteration (unsigned wrap-around) */
		runs_h_[r] = make_run(runs[r], first[r], ntl[r], log_tile,
			0u - runs[r].start_iter, fbase_h[r]);
		for (uint32_t t = 0; t < ntl[r]; t++) tile_run_h_[first[r] + t] = (uint16_t) r;
		base_h[r] = base;
		base += (uint32_t) runs[r].agents();
	}
	if (cfg.extra_tiles) free_tiles_.push_back({used_tiles_, cfg.extra_tiles});
	PP_CK(cudaMemcpyAsync(w_.runs, runs_h_.data(), nruns_cap * sizeof(RunDev), cudaMemcpyHostToDevice, s_));
	PP_CK(cudaMemcpyAsync(w_.tile_run, tile_run_h_.data(), tiles * 2, cudaMemcpyHostToDevice, s_));
	WorldCounters c{};
	tile_hi_ = used_tiles_;
	c.tile_hi = tile_hi_;
	PP_CK(cudaMemcpyAsync(w_.ctr, &c, sizeof(c), cudaMemcpyHostToDevice, s_));
	h2d_ += nruns_cap * sizeof(RunDev) + tiles * 2 + sizeof(c);

	/* Launch geometry. */
	lc_.sms = sms;
	lc_.cpt = (int) (T / ACT_THREADS);
	size_t act_smem = (size_t) act_cap * 20 + (size_t) T * 6;
	PP_CK(set_act_smem_limits(act_smem));
	PP_CK(set_step_smem_limits(act_smem));
	int occ_sort = occupancy_sort((int) d);
	if (occ_sort < 1) occ_sort = 1;
	lc_.sort_blocks = sms * occ_sort;
	lc_.move_blocks = (int) std::max<uint64_t>(1, std::min<uint64_t>((tiles + 7) / 8, (uint64_t) sms * 8));
	lc_.offs_blocks = sms * 8;
	lc_.finish_blocks = (int) std::min<uint64_t>(tiles, (uint64_t) sms * 2);
	lc_.act_tiles = (int) std::max<uint32_t>(tile_hi_, 1);

	/* Initial state: grass, then every run's agents in creation order into
	 * B at the run's base; fused pipeline: bucketed by tile and moved
	 * once; sort pipeline: sorted by cell into the region buffer, the
	 * tiles' regions and dense bases (runs occupy increasing cell ranges,
	 * so either way each run's agents stay at its base); stats row 0. */
	std::vector<PPStatistics> resumed_row0(runs.size());
	for (size_t r = 0; r < runs.size(); r++) {
		if (runs[r].init_val) {
			rc = load_run_state(runs[r], runs_h_[r], base_h[r], &resumed_row0[r]);
			if (rc) return rc;
			continue;
		}
		rc = cuda_status(enqueue_init_grass(w_, runs_h_[r], (uint32_t) r, 0, s_));
		if (rc) return rc;
		rc = cuda_status(enqueue_init_agents(w_, runs_h_[r], (uint32_t) r, 0,
			w_.kB, w_.vB, base_h[r],
			runs[r].p.init_sheep, runs[r].p.init_wolves, s_));
		if (rc) return rc;
	}
	if (w_.fused) {
		/* bucketed by tile; the first move of every agent into the group
		 * buffer the first act reads */
		rc = place_bucketed(base, 0, (uint32_t) tiles, 0);
		if (rc) return rc;
	} else {
		rc = sort_into(base, w_.kR, w_.vR);
		if (rc) return rc;
		rc = cuda_status(enqueue_regions_from_sorted(w_, lc_, w_.kR, 0, (uint32_t) tiles, 0, s_));
		if (rc) return rc;
	}
	/* row 0: summed by the init kernels, or the resumed state's */
	for (size_t r = 0; r < runs.size(); r++) {
		if (!runs[r].init_val) continue;
		PP_CK(cudaMemcpyAsync(&w_.ring[r], &resumed_row0[r], sizeof(PPStatistics),
			cudaMemcpyHostToDevice, s_));
		h2d_ += sizeof(PPStatistics);
	}
	for (size_t r = 0; r < runs.size(); r++) {
		rc = cuda_status(enqueue_focal_init(w_, (uint32_t) r, 0, runs[r].start_iter, s_));
		if (rc) return rc;
	}
	giter_ = 0;
	/* the graph of graph_iters iterations is captured by the first call
	 * that runs that many in a row, so a short job never pays for it */
	graph_iters_ = cfg.graph_iters;
	PP_CK(cudaStreamSynchronize(s_));
	return PP_SUCCESS;
}

int World::load_run_state(const RunSpec &spec, const RunDev &run, uint32_t base,
	PPStatistics *row0)
{
	/* A resumed run: its agents (run-local cells, canonical order) into B at
	 * its base; its grass as regrowth iterations start_iter + countdown,
	 * each pending regrowth counted in the run's histogram; the stats of
	 * the state as its row 0. */
	const uint32_t n = spec.init_n, cells = run.ncells, T0 = spec.start_iter;
	const uint32_t fs = run.restart + 1;
	std::vector<uint32_t> kc(n);
	PPStatistics st{};
	for (uint32_t i = 0; i < n; i++) {
		if (spec.init_cell[i] >= cells) return PP_INVALID_ARGS;
		if (i && spec.init_cell[i] < spec.init_cell[i - 1]) return PP_INVALID_ARGS;
		const uint32_t v = spec.init_val[i], e = v & ENERGY_MASK;
		if (e > run.emask) return PP_INVALID_ARGS;
		kc[i] = run.cbase + spec.init_cell[i];
		if (v & TYPE_BIT) { st.wolves++; st.wolves_en += e; }
		else { st.sheep++; st.sheep_en += e; }
	}
	std::vector<uint16_t> g(cells);
	std::vector<uint32_t> hist(fs, 0);
	for (uint32_t c = 0; c < cells; c++) {
		const uint32_t cd = spec.init_grass[c];
		if (cd > run.restart) return PP_INVALID_ARGS;
		g[c] = (uint16_t) (T0 + cd);
		if (cd) hist[(T0 + cd) % fs]++;
		else st.grass++;
		st.grass_en += cd;
	}
	*row0 = st;
	if (n) {
		PP_CK(cudaMemcpyAsync(w_.kB + base, kc.data(), (size_t) n * 4, cudaMemcpyHostToDevice, s_));
		PP_CK(cudaMemcpyAsync(w_.vB + base, spec.init_val, (size_t) n * 4, cudaMemcpyHostToDevice, s_));
	}
	PP_CK(cudaMemsetAsync(w_.grass + run.cbase, 0,
		((size_t) run.n_tiles << w_.log_tile) * sizeof(uint16_t), s_));
	PP_CK(cudaMemcpyAsync(w_.grass + run.cbase, g.data(), (size_t) cells * 2,
		cudaMemcpyHostToDevice, s_));
	PP_CK(cudaMemcpyAsync(w_.fring + run.fbase, hist.data(), (size_t) fs * 4,
		cudaMemcpyHostToDevice, s_));
	/* the host vectors go out of scope: wait for the copies */
	PP_CK(cudaStreamSynchronize(s_));
	h2d_ += (uint64_t) n * 8 + (uint64_t) cells * 2 + (uint64_t) fs * 4;
	return PP_SUCCESS;
}

int World::sort_into(uint32_t n, uint32_t *dst_k, uint32_t *dst_v)
{
	/* Stable radix sort of B[0, n) by the whole cell key (every region is a
	 * run of cell-sorted lists) on the world's counters, then a copy to
	 * dst; leaves fresh epochs, tickets and histograms. */
	PP_CK(cudaMemcpyAsync(&w_.ctr->aux_n, &n, 4, cudaMemcpyHostToDevice, s_));
	h2d_ += 4;
	if (n) {
		const uint32_t kb = w_.key_bits;
		const uint32_t passes = (kb + 7) / 8;
		uint32_t d = (kb + passes - 1) / passes;
		if (d < 5) d = 5;
		PP_CK(launch_radix_hist(w_.kB, &w_.ctr->aux_n, w_.hist, d, passes,
			lc_.move_blocks, s_));
		uint32_t *ki = w_.kB, *vi = w_.vB, *ko = w_.kC, *vo = w_.vC;
		for (uint32_t p = 0; p < passes; p++) {
			PP_CK(launch_radix_pass(ki, vi, ko, vo, w_.hist + p * 256, w_.lb_sort,
				w_.ctr, &w_.ctr->aux_n, p, p * d, d, lc_.sort_blocks, s_));
			std::swap(ki, ko);
			std::swap(vi, vo);
		}
		PP_CK(cudaMemcpyAsync(dst_k, ki, (size_t) n * 4, cudaMemcpyDeviceToDevice, s_));
		PP_CK(cudaMemcpyAsync(dst_v, vi, (size_t) n * 4, cudaMemcpyDeviceToDevice, s_));
	}
	PP_CK(enqueue_after_sort(w_.ctr, w_.hist, s_));
	return PP_SUCCESS;
}

int World::place_bucketed(uint32_t n, uint32_t first, uint32_t count,
	uint32_t out_base)
{
	/* the n agents of B (creation order, all in tiles [first, first +
	 * count)) bucketed by tile with their creation indices (no sort:
	 * the first move orders each cell's agents), fresh look-back epochs as
	 * after a sort, the first move of those tiles' agents into the group
	 * buffer from out_base on, then the dense input bases of the next act */
	PP_CK(cudaMemsetAsync(w_.tile_off + first, 0, ((size_t) count + 1) * 4, s_));
	PP_CK(enqueue_bucket_agents(w_, n, first, count, s_));
	PP_CK(enqueue_after_sort(w_.ctr, w_.hist, s_));
	PP_CK(enqueue_move_groups(w_, lc_, first, count, out_base, s_));
	PP_CK(enqueue_fused_bases(w_, lc_, s_));
	return PP_SUCCESS;
}

cudaError_t World::enqueue_one(const cudaEvent_t *marks)
{
	return w_.fused ? enqueue_iteration_fused(w_, lc_, s_, marks)
		: enqueue_iteration(w_, lc_, s_, marks);
}

void World::drop_graph()
{
	if (gexec_) { cudaGraphExecDestroy(gexec_); gexec_ = nullptr; }
	if (graph_) { cudaGraphDestroy(graph_); graph_ = nullptr; }
}

int World::build_graph()
{
	drop_graph();
	PP_CK(cudaStreamBeginCapture(s_, cudaStreamCaptureModeThreadLocal));
	for (uint32_t i = 0; i < graph_iters_; i++) {
		cudaError_t e = enqueue_one();
		if (e != cudaSuccess) {
			cudaGraph_t g;
			cudaStreamEndCapture(s_, &g);
			if (g) cudaGraphDestroy(g);
			return cuda_status(e);
		}
	}
	PP_CK(cudaStreamEndCapture(s_, &graph_));
	PP_CK(cudaGraphInstantiate(&gexec_, graph_, 0));
	return PP_SUCCESS;
}

int World::prepare_graph(uint32_t n)
{
	PP_CK(cudaSetDevice(device_));
	if (graph_iters_ && !gexec_ && n >= graph_iters_) return build_graph();
	return PP_SUCCESS;
}

int World::enqueue(uint32_t n)
{
	PP_CK(cudaSetDevice(device_));
	/* iterations run in stretches that end on multiples of REBASE, where
	 * the grass regrowth iterations are re-based (16-bit wrap-around) */
	uint32_t done = 0;
	while (done < n) {
		uint32_t to_rebase = REBASE - (giter_ % REBASE);
		uint32_t stretch = std::min(n - done, to_rebase);
		uint32_t k = 0;
		if (graph_iters_ && stretch >= graph_iters_) {
			if (!gexec_) {
				const int rc = build_graph();
				if (rc) return rc;
			}
			while (stretch - k >= graph_iters_) {
				PP_CK(cudaGraphLaunch(gexec_, s_));
				k += graph_iters_;
			}
		}
		for (; k < stretch; k++) PP_CK(enqueue_one());
		giter_ += stretch;
		done += stretch;
		if (giter_ % REBASE == 0) PP_CK(enqueue_grass_rebase(w_, lc_, s_));
	}
	if (n) {
		release_pending();
		adm_used_ = 0;   /* the act rewrote every region below 2 * cap */
	}
	return PP_SUCCESS;
}

int World::sync_check()
{
	PP_CK(cudaSetDevice(device_));
	PP_CK(cudaStreamSynchronize(s_));
	uint32_t err = 0;
	PP_CK(cudaMemcpy(&err, &w_.ctr->err, 4, cudaMemcpyDeviceToHost));
	d2h_ += 4;
	if (err & ERRF_TIMEOUT) return PP_ERR_TIMEOUT;
	if (err & ERRF_OVERFLOW) return PP_OUT_OF_RESOURCES;
	return PP_SUCCESS;
}

uint32_t World::n_agents_dev()
{
	uint32_t n = 0;
	cudaSetDevice(device_);
	cudaStreamSynchronize(s_);
	cudaMemcpy(&n, &w_.ctr->n_agents, 4, cudaMemcpyDeviceToHost);
	return n;
}

int World::read_rows(uint32_t r, uint32_t g0, uint32_t g1, PPStatistics *out)
{
	if (g1 < g0) return PP_SUCCESS;
	PP_CK(cudaSetDevice(device_));
	const uint32_t R = w_.ring_rows;
	const size_t pitch = (size_t) w_.nruns_cap * sizeof(PPStatistics);
	uint32_t g = g0;
	while (g <= g1) {
		uint32_t pos = g % R;
		uint32_t cnt = std::min<uint32_t>(g1 - g + 1, R - pos);
		PP_CK(cudaMemcpy2DAsync(out + (g - g0), sizeof(PPStatistics),
			&w_.ring[(size_t) pos * w_.nruns_cap + r], pitch,
			sizeof(PPStatistics), cnt, cudaMemcpyDeviceToHost, s_));
		d2h_ += (uint64_t) cnt * sizeof(PPStatistics);
		g += cnt;
	}
	PP_CK(cudaStreamSynchronize(s_));
	return PP_SUCCESS;
}

int World::read_ring(uint32_t g0, uint32_t g1, uint32_t nslots, PPStatistics *out)
{
	if (g1 < g0 || nslots == 0) return PP_SUCCESS;
	PP_CK(cudaSetDevice(device_));
	const uint32_t R = w_.ring_rows;
	const size_t pitch = (size_t) w_.nruns_cap * sizeof(PPStatistics);
	uint32_t g = g0;
	while (g <= g1) {
		uint32_t pos = g % R;
		uint32_t cnt = std::min<uint32_t>(g1 - g + 1, R - pos);
		PP_CK(cudaMemcpy2DAsync(out + (size_t) (g - g0) * nslots,
			nslots * sizeof(PPStatistics), &w_.ring[(size_t) pos * w_.nruns_cap],
			pitch, nslots * sizeof(PPStatistics), cnt, cudaMemcpyDeviceToHost, s_));
		d2h_ += (uint64_t) cnt * nslots * sizeof(PPStatistics);
		g += cnt;
	}
	PP_CK(cudaStreamSynchronize(s_));
	return PP_SUCCESS;
}

int World::get_state(uint32_t *cell, uint32_t *en, uint32_t n_max,
	uint32_t *n_out, uint16_t *grass, uint32_t r)
{
	PP_CK(cudaSetDevice(device_));
	PP_CK(cudaStreamSynchronize(s_));
	if (w_.fused) {
		int rc = get_state_fused(cell, en, n_max, n_out, r);
		if (rc) return rc;
		cell = nullptr;
		en = nullptr;
	}
	uint32_t n = 0, m = 0;
	if (!w_.fused) {
	PP_CK(cudaMemcpy(&n, &w_.ctr->n_agents, 4, cudaMemcpyDeviceToHost));
	if (n_out) *n_out = n;
	m = std::min(n, n_max);
	PP_CK(enqueue_compact(w_, lc_, w_.kA, w_.vA, s_));
	PP_CK(cudaStreamSynchronize(s_));
	if (cell && m) PP_CK(cudaMemcpy(cell, w_.kA, (size_t) m * 4, cudaMemcpyDeviceToHost));
	if (en && m) PP_CK(cudaMemcpy(en, w_.vA, (size_t) m * 4, cudaMemcpyDeviceToHost));
	}
	if (grass) {
		/* stored regrowth iterations -> countdowns of the current iteration */
		const RunDev &run = runs_h_[r];
		PP_CK(cudaMemcpy(grass, w_.grass + run.cbase,
			(size_t) run.ncells * 2, cudaMemcpyDeviceToHost));
		const uint16_t t16 = (uint16_t) (giter_ - run.start_giter);
		for (uint32_t c = 0; c < run.ncells; c++) {
			const int32_t dd = (int16_t) (uint16_t) (grass[c] - t16);
			grass[c] = (uint16_t) (dd > 0 ? dd : 0);
		}
	}
	if (cell && m) {
		/* Report cells relative to the run's grid. */
		uint32_t cb = runs_h_[r].cbase;
		for (uint32_t i = 0; i < m; i++) cell[i] -= cb;
	}
	return PP_SUCCESS;
}

int World::get_state_fused(uint32_t *cell, uint32_t *en, uint32_t n_max,
	uint32_t *n_out, uint32_t r)
{
	/* The state after the last act is the group buffer of the next parity:
	 * every record of the run's tiles' inboxes (moved ones with their
	 * direction, dead and parked ones in place), mapped back to the cell
	 * before the move and the energy before it, in canonical order (cell,
	 * rank in the cell's list). */
	const RunDev &run = runs_h_[r];
	const uint32_t p = (giter_ + 1) & 1;
	const uint32_t T = 1u << w_.log_tile;
	const size_t nt = run.n_tiles;
	std::vector<uint32_t> inn(nt);
	std::vector<uint2> ent(nt * IBX);
	if (nt) {
		const size_t ib = (size_t) p * w_.n_tiles + run.first_tile;
		PP_CK(cudaMemcpy(inn.data(), w_.inbox_n + ib, nt * 4, cudaMemcpyDeviceToHost));
		PP_CK(cudaMemcpy(ent.data(), w_.inbox + ib * IBX, nt * IBX * sizeof(uint2),
			cudaMemcpyDeviceToHost));
	}
	/* the group buffer up to the end of the last listed group */
	uint64_t top = 0;
	for (size_t q = 0; q < nt; q++)
		for (uint32_t i = 0; i < std::min(inn[q], IBX); i++) {
			const uint2 e = ent[q * IBX + i];
			top = std::max<uint64_t>(top, (uint64_t) e.x + (e.y & ~GROUP_GRAVE));
		}
	top = std::min<uint64_t>(top, 3ull * w_.cap);
	std::vector<uint32_t> kg(top), vg(top);
	if (top) {
		PP_CK(cudaMemcpy(kg.data(), p ? w_.kG1 : w_.kG0, (size_t) top * 4, cudaMemcpyDeviceToHost));
		PP_CK(cudaMemcpy(vg.data(), p ? w_.vG1 : w_.vG0, (size_t) top * 4, cudaMemcpyDeviceToHost));
	}
	d2h_ += (uint64_t) top * 8 + nt * (4 + IBX * sizeof(uint2)) + 4;
	struct Rec { uint32_t cell, rank, val; };
	std::vector<Rec> recs;
	for (size_t q = 0; q < nt; q++) {
		const uint32_t tile = run.first_tile + (uint32_t) q;
		const uint32_t nin = std::min(inn[q], IBX);
		for (uint32_t i = 0; i < nin; i++) {
			const uint2 e = ent[q * IBX + i];
			const uint32_t c = e.y & ~GROUP_GRAVE;
			for (uint32_t a = e.x; a < e.x + c && a < top; a++) {
				const uint32_t key = kg[a], val = vg[a];
				const uint32_t code = (key >> REC_DIR_SHIFT) & 7u;
				const uint32_t lr = (tile << w_.log_tile) + (key & (T - 1)) - run.cbase;
				Rec rc;
				rc.rank = key >> REC_RANK_SHIFT;
				if (code <= 4) {
					const uint32_t y = lr / run.gx, x = lr - y * run.gx;
					rc.cell = (uint32_t) ((int64_t) lr + src_offset(code, x, y, run.gx, run.gy));
					rc.val = val + 1;
				} else {
					rc.cell = lr;
					rc.val = val;
				}
				recs.push_back(rc);
			}
		}
	}
	std::sort(recs.begin(), recs.end(), [](const Rec &a, const Rec &b) {
		return a.cell != b.cell ? a.cell < b.cell : a.rank < b.rank;
	});
	const uint32_t n = (uint32_t) recs.size();
	if (n_out) *n_out = n;
	const uint32_t m = std::min(n, n_max);
	for (uint32_t i = 0; i < m; i++) {
		if (cell) cell[i] = recs[i].cell;
		if (en) en[i] = recs[i].val;
	}
	return PP_SUCCESS;
}

int World::profile(uint32_t n, pp_kernel_prof *prof, double *agent_steps)
{
	PP_CK(cudaSetDevice(device_));
	const uint32_t P = w_.passes;
	std::vector<cudaEvent_t> ev(P + 5);
	for (auto &e : ev) PP_CK(cudaEventCreate(&e));
	static const char *names[5] = {"move", "radix_pass", "offsets", "act", "finish"};
	for (int k = 0; k < 5; k++) {
		memset(&prof[k], 0, sizeof(prof[k]));
		snprintf(prof[k].name, sizeof(prof[k].name), "%s", names[k]);
	}
	uint64_t live_cells = 0;
	for (uint32_t r = 0; r < null_slot_; r++)
		if (runs_h_[r].active) live_cells += runs_h_[r].ncells;
	double steps = 0;
	int rc = PP_SUCCESS;
	for (uint32_t it = 0; it < n && rc == PP_SUCCESS && w_.fused; it++) {
		uint32_t n_before = 0, n_after = 0;
		PP_CK(cudaMemcpyAsync(&n_before, &w_.ctr->n_agents, 4, cudaMemcpyDeviceToHost, s_));
		PP_CK(cudaStreamSynchronize(s_));
		rc = cuda_status(enqueue_one(ev.data()));
		if (rc) break;
		PP_CK(cudaMemcpyAsync(&n_after, &w_.ctr->n_agents, 4, cudaMemcpyDeviceToHost, s_));
		PP_CK(cudaStreamSynchronize(s_));
		giter_++;
		float ms;
		PP_CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
		prof[3].launches++; prof[3].total_ms += ms;
		/* act+move: the tile's records in, survivors and newborns out as
		 * moved records, the regrowth word of each occupied cell (at most
		 * one read per agent) */
		prof[3].bytes += 10.0 * n_before + 8.0 * n_after;
		PP_CK(cudaEventElapsedTime(&ms, ev[1], ev[2]));
		prof[4].launches++; prof[4].total_ms += ms;
		prof[4].bytes += 48.0 * w_.n_tiles;
		steps += n_before;
	}
	for (uint32_t it = 0; it < n && rc == PP_SUCCESS && !w_.fused; it++) {
		uint32_t n_before = 0, n_live = 0, n_after = 0;
		PP_CK(cudaMemcpyAsync(&n_before, &w_.ctr->n_agents, 4, cudaMemcpyDeviceToHost, s_));
		PP_CK(cudaStreamSynchronize(s_));
		rc = cuda_status(enqueue_one(ev.data()));
		if (rc) break;
		PP_CK(cudaMemcpyAsync(&n_live, &w_.tile_off[w_.n_tiles], 4, cudaMemcpyDeviceToHost, s_));
		PP_CK(cudaMemcpyAsync(&n_after, &w_.ctr->n_agents, 4, cudaMemcpyDeviceToHost, s_));
		PP_CK(cudaStreamSynchronize(s_));
		giter_++;
		float ms;
		PP_CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
		prof[0].launches++; prof[0].total_ms += ms;
		prof[0].bytes += 16.0 * n_before;
		for (uint32_t p = 0; p < P; p++) {
			PP_CK(cudaEventElapsedTime(&ms, ev[1 + p], ev[2 + p]));
			prof[1].launches++; prof[1].total_ms += ms;
			prof[1].bytes += 16.0 * n_before;
		}
		PP_CK(cudaEventElapsedTime(&ms, ev[1 + P], ev[2 + P]));
		prof[2].launches++; prof[2].total_ms += ms;
		prof[2].bytes += 4.0 * n_before + 4.0 * (w_.n_tiles + 1);
		PP_CK(cudaEventElapsedTime(&ms, ev[2 + P], ev[3 + P]));
		prof[3].launches++; prof[3].total_ms += ms;
		/* act: sorted agents in, survivors and newborns out, the regrowth
		 * word of each occupied cell (at most one per agent) */
		prof[3].bytes += 10.0 * n_live + 8.0 * n_after;
		PP_CK(cudaEventElapsedTime(&ms, ev[3 + P], ev[4 + P]));
		prof[4].launches++; prof[4].total_ms += ms;
		prof[4].bytes += 48.0 * w_.n_tiles;
		steps += n_before;
	}
	for (auto &e : ev) cudaEventDestroy(e);
	if (agent_steps) *agent_steps = steps;
	if (rc) return rc;
	return sync_check();
}

int World::update_tile_hi()
{
	/* tiles of active runs and of retired runs still in quarantine */
	uint32_t hi = 0;
	for (uint32_t r = 0; r < null_slot_; r++)
		if (runs_h_[r].active) hi = std::max(hi, runs_h_[r].first_tile + runs_h_[r].n_tiles);
	for (auto &pt : pending_tiles_) hi = std::max(hi, pt.first.first + pt.first.second);
	if (hi == tile_hi_) return PP_SUCCESS;
	tile_hi_ = hi;
	lc_.act_tiles = (int) std::max<uint32_t>(tile_hi_, 1);
	PP_CK(cudaMemcpyAsync(&w_.ctr->tile_hi, &tile_hi_, 4, cudaMemcpyHostToDevice, s_));
	PP_CK(cudaStreamSynchronize(s_));
	h2d_ += 4;
	/* the captured iterations carry the old grid: captured again when next
	 * needed */
	drop_graph();
	return PP_SUCCESS;
}

bool World::fits(const RunSpec &spec) const
{
	uint32_t need = ceil_div((uint64_t) spec.p.grid_x * spec.p.grid_y,
		1u << w_.log_tile);
	bool tiles_ok = false;
	for (auto &f : free_tiles_) if (f.second >= need) { tiles_ok = true; break; }
	bool slot_ok = false;
	for (uint32_t r = 0; r < null_slot_; r++)
		if (!runs_h_[r].active) { slot_ok = true; break; }
	return tiles_ok && slot_ok;
}

int World::admit(const RunSpec &spec, uint32_t *slot_out)
{
	pp::NvtxRange nvtx_range("admit");
	PP_CK(cudaSetDevice(device_));
	uint32_t need = ceil_div((uint64_t) spec.p.grid_x * spec.p.grid_y,
		1u << w_.log_tile);
	int fi = -1;
	for (size_t i = 0; i < free_tiles_.size(); i++)
		if (free_tiles_[i].second >= need) { fi = (int) i; break; }
	uint32_t slot = null_slot_;
	for (uint32_t r = 0; r < null_slot_; r++)
		if (!runs_h_[r].active) { slot = r; break; }
	if (fi < 0 || slot == null_slot_) return PP_OUT_OF_RESOURCES;
	uint32_t first = free_tiles_[fi].first;
	free_tiles_[fi].first += need;
	free_tiles_[fi].second -= need;
	if (free_tiles_[fi].second == 0) free_tiles_.erase(free_tiles_.begin() + fi);

	PP_CK(cudaStreamSynchronize(s_));
	uint32_t n = 0;
	PP_CK(cudaMemcpy(&n, &w_.ctr->n_agents, 4, cudaMemcpyDeviceToHost));
	uint32_t n0 = spec.p.init_sheep + spec.p.init_wolves;
	if ((uint64_t) n + n0 > w_.cap || (uint64_t) adm_used_ + n0 > w_.cap) {
		free_tiles_.push_back({first, need});
		return PP_OUT_OF_RESOURCES;
	}
	const uint32_t fbase = fslot_base_ + slot * FSLOT;
	RunDev run = make_run(spec, first, need, w_.log_tile, giter_, fbase);
	PP_CK(cudaMemsetAsync(w_.fring + fbase, 0, (spec.p.grass_restart + 1) * 4, s_));
	runs_h_[slot] = run;
	for (uint32_t t = 0; t < need; t++) tile_run_h_[first + t] = (uint16_t) slot;
	PP_CK(cudaMemcpyAsync(&w_.runs[slot], &run, sizeof(RunDev), cudaMemcpyHostToDevice, s_));
	PP_CK(cudaMemcpyAsync(&w_.tile_run[first], &tile_run_h_[first], need * 2, cudaMemcpyHostToDevice, s_));
	int rc0 = update_tile_hi();
	if (rc0) return rc0;
	uint32_t row = giter_ % w_.ring_rows;
	PP_CK(cudaMemsetAsync(&w_.ring[(size_t) row * w_.nruns_cap + slot], 0, sizeof(PPStatistics), s_));
	/* Grass of its tiles; its agents bucketed by tile (fused pipeline) or
	 * sorted by cell (sort pipeline), and moved in. The other runs' agents
	 * stay in place: draws never depend on positions. */
	int rc = cuda_status(enqueue_init_grass(w_, run, slot, row, s_));
	if (rc) return rc;
	rc = cuda_status(enqueue_init_agents(w_, run, slot, row, w_.kB, w_.vB, 0,
		spec.p.init_sheep, spec.p.init_wolves, s_));
	if (rc) return rc;
	if (w_.fused) {
		/* bucketed into A, moved into the group buffer the next act reads */
		rc = place_bucketed(n0, first, need, 2 * w_.cap + adm_used_);
		if (rc) return rc;
		adm_used_ += n0;
		PP_CK(cudaStreamSynchronize(s_));
		rc = cuda_status(enqueue_focal_init(w_, slot, row, 0, s_));
		if (rc) return rc;
	} else {
		/* The agents go to the admission area of the region buffer (after
		 * the 2 * cap slots the act writes), as the regions of the run's
		 * tiles. */
		const uint32_t adm = 2 * w_.cap + adm_used_;
		rc = sort_into(n0, w_.kR + adm, w_.vR + adm);
		if (rc) return rc;
		rc = cuda_status(enqueue_regions_from_sorted(w_, lc_, w_.kR + adm, first, need, adm, s_));
		if (rc) return rc;
		adm_used_ += n0;
		rc = cuda_status(enqueue_focal_init(w_, slot, row, 0, s_));
		if (rc) return rc;
	}
	h2d_ += sizeof(RunDev) + need * 2;
	d2h_ += 4;
	*slot_out = slot;
	return PP_SUCCESS;
}

int World::read_focal(uint32_t r, FocalDev *out)
{
	PP_CK(cudaSetDevice(device_));
	PP_CK(cudaStreamSynchronize(s_));
	PP_CK(cudaMemcpy(out, &w_.focal[r], sizeof(FocalDev), cudaMemcpyDeviceToHost));
	d2h_ += sizeof(FocalDev);
	return PP_SUCCESS;
}

int World::retire(uint32_t slot)
{
	PP_CK(cudaSetDevice(device_));
	if (slot >= null_slot_ || !runs_h_[slot].active) return PP_INVALID_ARGS;
	RunDev &run = runs_h_[slot];
	uint32_t first = run.first_tile, cnt = run.n_tiles;
	run.active = 0;
	/* The run's agents die in the next move (inactive run). Its tiles go
	 * back to the free list, mapped to the null slot. */
	PP_CK(cudaMemcpyAsync(&w_.runs[slot], &run, sizeof(RunDev), cudaMemcpyHostToDevice, s_));
	for (uint32_t t = 0; t < cnt; t++) tile_run_h_[first + t] = (uint16_t) null_slot_;
	PP_CK(cudaMemcpyAsync(&w_.tile_run[first], &tile_run_h_[first], (size_t) cnt * 2,
		cudaMemcpyHostToDevice, s_));
	h2d_ += sizeof(RunDev) + (size_t) cnt * 2;
	/* The run's last agents are still in the agent array; they die in the
	 * next move (their tiles now map to the inactive null slot). Until an
	 * iteration has run, the tiles must not be handed to another run. */
	pending_tiles_.push_back({{first, cnt}, giter_});
	return PP_SUCCESS;
}

void World::release_pending()
{
	bool any = false;
	for (size_t i = 0; i < pending_tiles_.size();) {
		if (pending_tiles_[i].second < giter_) {
			free_tiles_.push_back(pending_tiles_[i].first);
			pending_tiles_.erase(pending_tiles_.begin() + i);
			any = true;
		} else {
			i++;
		}
	}
	if (!any) return;
	update_tile_hi();
	std::sort(free_tiles_.begin(), free_tiles_.end());
	std::vector<std::pair<uint32_t, uint32_t>> merged;
	for (auto &f : free_tiles_) {
		if (!merged.empty() && merged.back().first + merged.back().second == f.first)
			merged.back().second += f.second;
		else merged.push_back(f);
	}
	free_tiles_.swap(merged);
}

} /* namespace pp */

/* ==================================================================== */
/* C ABI                                                                 */
/* ==================================================================== */

using namespace pp;

extern "C" int pp_params_check(const PPParameters *p, char *errmsg, size_t errlen);

struct pp_sim {
	World world;
	PPParameters params;
	uint64_t seed;
	PPStatistics stats0;
	uint32_t iter0 = 0;     /* iteration the simulation was restored at */
	uint32_t agent_size = 0; /* pp_opts.agent_size it was created with */
};

extern "C" void pp_opts_default(pp_opts *o)
{
	memset(o, 0, sizeof(*o));
	o->device = 0;
	o->max_agents = 0;
	o->tile_cells = 0;
	o->sort_digit_bits = 0;
	o->use_graph = 1;
	o->sort_pipeline = 0;
	o->ss_from = 1000;
}

/* A simulation from parameters and a seed, or from a saved state (spec0's
 * init arrays and start iteration). */
static int sim_create(const PPParameters *params, uint64_t seed,
	const pp_opts *opts, const RunSpec *spec0, pp_sim **out)
{
	pp::NvtxRange nvtx_range("pp_sim_create");
	if (!params || !out) return PP_INVALID_ARGS;
	*out = nullptr;
	PPParameters p = *params;
	p.grid_xy = p.grid_x * p.grid_y;
	int rc = pp_params_check(&p, nullptr, 0);
	if (rc) return rc;
	pp_opts o;
	if (opts) o = *opts;
	else pp_opts_default(&o);
	uint32_t ebits = 30;
	rc = agent_energy_bits(o.agent_size, p, &ebits);
	if (rc) return rc;
	pp_sim *sim = new (std::nothrow) pp_sim();
	if (!sim) return PP_OUT_OF_RESOURCES;
	sim->params = p;
	sim->seed = seed;
	sim->agent_size = o.agent_size;
	WorldConfig cfg;
	cfg.device = o.device;
	uint64_t n0 = (uint64_t) p.init_sheep + p.init_wolves;
	if (spec0) n0 = std::max<uint64_t>(n0, spec0->init_n);
	uint64_t cap = o.max_agents ? o.max_agents
		: std::max<uint64_t>(std::max<uint64_t>(4 * n0, 1024), 16777216ull);
	cfg.cap = (uint32_t) std::min<uint64_t>(cap, 0x7fffffffu);
	cfg.tile_cells = o.tile_cells;
	cfg.digit_bits = o.sort_digit_bits;
	cfg.graph_iters = o.use_graph ? 32 : 0;
	cfg.fused = o.sort_pipeline == 0;
	if (o.autotune && o.tile_cells == 0) {
		pp_tuning tu;
		rc = pp_autotune(&p, seed, cfg.cap, o.device, &tu);
		if (rc) {
			delete sim;
			return rc;
		}
		cfg.tile_cells = tu.tile_cells;
		cfg.fused = tu.sort_pipeline == 0;
		if (tu.sort_digit_bits) cfg.digit_bits = tu.sort_digit_bits;
	}
	std::vector<RunSpec> runs(1);
	if (spec0) runs[0] = *spec0;
	runs[0].p = p;
	runs[0].seed = seed;
	runs[0].iters = 0xffffffffu;
	runs[0].ss_from = o.ss_from;
	runs[0].energy_bits = ebits;
	sim->iter0 = spec0 ? spec0->start_iter : 0;
	rc = sim->world.create(runs, cfg);
	if (rc == PP_SUCCESS) rc = sim->world.read_rows(0, 0, 0, &sim->stats0);
	if (rc) {
		delete sim;
		cudaGetLastError();
		return rc;
	}
	*out = sim;
	return PP_SUCCESS;
}

extern "C" int pp_sim_create(const PPParameters *params, uint64_t seed,
	const pp_opts *opts, pp_sim **out)
{
	return sim_create(params, seed, opts, nullptr, out);
}

/* Snapshot file: magic, parameters, seed, iteration, agent count, agent
 * size (pp_opts.agent_size), then the agents' run-local cells and type |
 * energy words in canonical order and the grid's grass countdowns (native
 * byte order). Files of the first version (magic ...01) have no agent size
 * field; they restore with the caller's. */
static const char SNAP_MAGIC[8] = {'P', 'P', 'S', 'N', 'A', 'P', '0', '2'};
static const char SNAP_MAGIC_V1[8] = {'P', 'P', 'S', 'N', 'A', 'P', '0', '1'};

extern "C" int pp_sim_snapshot_save(pp_sim *sim, const char *path)
{
	pp::NvtxRange nvtx_range("pp_sim_snapshot_save");
	if (!sim || !path) return PP_INVALID_ARGS;
	World &w = sim->world;
	uint32_t n = 0;
	int rc = w.get_state(nullptr, nullptr, 0, &n, nullptr, 0);
	if (rc) return rc;
	const PPParameters &p = sim->params;
	std::vector<uint32_t> cell(std::max<uint32_t>(n, 1)), en(std::max<uint32_t>(n, 1));
	std::vector<uint16_t> grass((size_t) p.grid_x * p.grid_y);
	uint32_t n2 = 0;
	rc = w.get_state(cell.data(), en.data(), n, &n2, grass.data(), 0);
	if (rc) return rc;
	if (n2 != n) return PP_LIBRARY_ERROR;
	const uint32_t iter = sim->iter0 + w.giter();
	FILE *f = fopen(path, "wb");
	if (!f) return PP_UNABLE_SAVE_STATS;
	bool ok = fwrite(SNAP_MAGIC, 1, 8, f) == 8
		&& fwrite(&p, sizeof(p), 1, f) == 1
		&& fwrite(&sim->seed, 8, 1, f) == 1
		&& fwrite(&iter, 4, 1, f) == 1
		&& fwrite(&n, 4, 1, f) == 1
		&& fwrite(&sim->agent_size, 4, 1, f) == 1
		&& (n == 0 || fwrite(cell.data(), 4, n, f) == n)
		&& (n == 0 || fwrite(en.data(), 4, n, f) == n)
		&& fwrite(grass.data(), 2, grass.size(), f) == grass.size();
	if (fclose(f) != 0) ok = false;
	return ok ? PP_SUCCESS : PP_UNABLE_SAVE_STATS;
}

extern "C" int pp_sim_restore(const char *path, const pp_opts *opts, pp_sim **out)
{
	if (!path || !out) return PP_INVALID_ARGS;
	*out = nullptr;
	FILE *f = fopen(path, "rb");
	if (!f) return PP_UNABLE_TO_OPEN_PARAMS_FILE;
	char magic[8];
	PPParameters p;
	uint64_t seed = 0;
	uint32_t iter = 0, n = 0;
	pp_opts o;
	if (opts) o = *opts;
	else pp_opts_default(&o);
	bool ok = fread(magic, 1, 8, f) == 8;
	const bool v1 = ok && memcmp(magic, SNAP_MAGIC_V1, 8) == 0;
	ok = ok && (v1 || memcmp(magic, SNAP_MAGIC, 8) == 0)
		&& fread(&p, sizeof(p), 1, f) == 1 && fread(&seed, 8, 1, f) == 1
		&& fread(&iter, 4, 1, f) == 1 && fread(&n, 4, 1, f) == 1
		&& (v1 || fread(&o.agent_size, 4, 1, f) == 1)
		&& p.grid_x > 0 && p.grid_y > 0 && p.grid_x <= 65535 && p.grid_y <= 65535
		&& n < 0x80000000u;
	std::vector<uint32_t> cell, en;
	std::vector<uint16_t> grass;
	if (ok) {
		cell.resize(std::max<uint32_t>(n, 1));
		en.resize(std::max<uint32_t>(n, 1));
		grass.resize((size_t) p.grid_x * p.grid_y);
		ok = (n == 0 || fread(cell.data(), 4, n, f) == n)
			&& (n == 0 || fread(en.data(), 4, n, f) == n)
			&& fread(grass.data(), 2, grass.size(), f) == grass.size();
	}
	fclose(f);
	if (!ok) return PP_INVALID_PARAMS_FILE;
	RunSpec spec;
	spec.init_cell = cell.data();
	spec.init_val = en.data();
	spec.init_grass = grass.data();
	spec.init_n = n;
	spec.start_iter = iter;
	return sim_create(&p, seed, &o, &spec, out);
}

void pp::focal_export(const FocalDev &f, pp_focal *out)
{
	memset(out, 0, sizeof(*out));
	for (int k = 0; k < 6; k++) {
		out->max[k] = f.mx[k];
		out->min[k] = f.mn[k];
		out->argmax[k] = f.amx[k];
		out->argmin[k] = f.amn[k];
		if (f.n) out->ss_mean[k] = f.sum[k] / f.n;
		if (f.n > 1) {
			const double var = (f.sq[k] - f.sum[k] * f.sum[k] / f.n) / (f.n - 1);
			out->ss_std[k] = var > 0 ? sqrt(var) : 0.0;
		}
	}
	out->ss_n = f.n;
}

extern "C" int pp_sim_focal(pp_sim *sim, pp_focal *out)
{
	if (!sim || !out) return PP_INVALID_ARGS;
	FocalDev f;
	int rc = sim->world.read_focal(0, &f);
	if (rc) return rc;
	focal_export(f, out);
	return PP_SUCCESS;
}

extern "C" int pp_sim_params(pp_sim *sim, PPParameters *out)
{
	if (!sim || !out) return PP_INVALID_ARGS;
	*out = sim->params;
	return PP_SUCCESS;
}

extern "C" int pp_sim_stats0(pp_sim *sim, PPStatistics *out)
{
	if (!sim || !out) return PP_INVALID_ARGS;
	*out = sim->stats0;
	return PP_SUCCESS;
}

extern "C" int pp_sim_step(pp_sim *sim, uint32_t n_iters, PPStatistics *out)
{
	pp::NvtxRange nvtx_range("pp_sim_step");
	if (!sim) return PP_INVALID_ARGS;
	World &w = sim->world;
	const uint32_t chunk_max = w.ring_rows() - 1;
	uint32_t done = 0;
	while (done < n_iters) {
		uint32_t chunk = std::min(n_iters - done, chunk_max);
		uint32_t g0 = w.giter();
		int rc = w.enqueue(chunk);
		if (rc) return rc;
		rc = w.sync_check();
		if (rc) return rc;
		if (out) {
			rc = w.read_rows(0, g0 + 1, g0 + chunk, out + done);
			if (rc) return rc;
		}
		done += chunk;
	}
	return PP_SUCCESS;
}

extern "C" int pp_sim_step_async(pp_sim *sim, uint32_t n_iters, void *dev_stats)
{
	if (!sim) return PP_INVALID_ARGS;
	World &w = sim->world;
	if (n_iters >= w.ring_rows()) return PP_INVALID_ARGS;
	uint32_t g0 = w.giter();
	int rc = w.enqueue(n_iters);
	if (rc) return rc;
	if (dev_stats && n_iters) {
		const uint32_t R = w.ring_rows();
		const size_t pitch = (size_t) w.dev().nruns_cap * sizeof(PPStatistics);
		uint32_t g = g0 + 1, g1 = g0 + n_iters;
		PPStatistics *dst = (PPStatistics *) dev_stats;
		while (g <= g1) {
			uint32_t pos = g % R;
			uint32_t cnt = std::min<uint32_t>(g1 - g + 1, R - pos);
			cudaError_t e = cudaMemcpy2DAsync(dst + (g - g0 - 1),
				sizeof(PPStatistics), &w.dev().ring[(size_t) pos * w.dev().nruns_cap],
				pitch, sizeof(PPStatistics), cnt, cudaMemcpyDeviceToDevice,
				w.stream());
			if (e != cudaSuccess) return cuda_status(e);
			g += cnt;
		}
	}
	return PP_SUCCESS;
}

extern "C" int pp_sim_sync(pp_sim *sim)
{
	if (!sim) return PP_INVALID_ARGS;
	return sim->world.sync_check();
}

extern "C" int pp_sim_info(pp_sim *sim, uint32_t *iter, uint32_t *n_agents,
	uint32_t *capacity)
{
	if (!sim) return PP_INVALID_ARGS;
	if (iter) *iter = sim->iter0 + sim->world.giter();
	if (n_agents) *n_agents = sim->world.n_agents_dev();
	if (capacity) *capacity = sim->world.dev().cap;
	return PP_SUCCESS;
}

extern "C" int pp_sim_get_state(pp_sim *sim, uint32_t *cell, uint32_t *en,
	uint32_t n_max, uint32_t *n_agents, uint16_t *grass)
{
	if (!sim) return PP_INVALID_ARGS;
	return sim->world.get_state(cell, en, n_max, n_agents, grass, 0);
}

extern "C" int pp_sim_profile(pp_sim *sim, uint32_t n_iters,
	pp_kernel_prof *prof, uint32_t n_prof, double *agent_steps)
{
	if (!sim || !prof || n_prof < 5) return PP_INVALID_ARGS;
	if (n_iters >= sim->world.ring_rows()) return PP_INVALID_ARGS;
	return sim->world.profile(n_iters, prof, agent_steps);
}

extern "C" int pp_sim_time(pp_sim *sim, uint32_t n_iters, float *ms)
{
	if (!sim || !ms) return PP_INVALID_ARGS;
	if (n_iters >= sim->world.ring_rows()) return PP_INVALID_ARGS;
	World &w = sim->world;
	cudaEvent_t a, b;
	PP_CK(cudaSetDevice(w.dev_index()));
	int rc = w.prepare_graph(n_iters);
	if (rc) return rc;
	PP_CK(cudaEventCreate(&a));
	PP_CK(cudaEventCreate(&b));
	PP_CK(cudaEventRecord(a, w.stream()));
	rc = w.enqueue(n_iters);
	PP_CK(cudaEventRecord(b, w.stream()));
	if (rc == PP_SUCCESS) rc = w.sync_check();
	if (rc == PP_SUCCESS) PP_CK(cudaEventElapsedTime(ms, a, b));
	cudaEventDestroy(a);
	cudaEventDestroy(b);
	return rc;
}

extern "C" int pp_sim_stats_range(pp_sim *sim, uint32_t first_iter,
	uint32_t n, PPStatistics *out)
{
	if (!sim || !out) return PP_INVALID_ARGS;
	World &w = sim->world;
	uint32_t g = w.giter();
	if (n == 0) return PP_SUCCESS;
	if (first_iter + n - 1 > g || g - first_iter >= w.ring_rows())
		return PP_INVALID_ARGS;
	return w.read_rows(0, first_iter, first_iter + n - 1, out);
}

extern "C" int pp_sim_io_bytes(pp_sim *sim, uint64_t *h2d, uint64_t *d2h)
{
	if (!sim) return PP_INVALID_ARGS;
	if (h2d) *h2d = sim->world.h2d_;
	if (d2h) *d2h = sim->world.d2h_;
	return PP_SUCCESS;
}

extern "C" void *pp_sim_stream(pp_sim *sim)
{
	return sim ? (void *) sim->world.stream() : nullptr;
}

extern "C" int pp_sim_destroy(pp_sim *sim)
{
	delete sim;
	return PP_SUCCESS;
}

/* ---------------- kernel-level entry points ---------------- */

namespace {

struct DevBuf {
	void *p = nullptr;
	~DevBuf() { if (p) cudaFree(p); }
	cudaError_t alloc(size_t n) { return cudaMalloc(&p, n ? n : 16); }
	template <typename T> T *as() { return (T *) p; }
};

} /* namespace */

extern "C" int pp_philox_fill(uint32_t c0, uint32_t c1, uint32_t c2,
	uint32_t c3, uint32_t k0, uint32_t k1, uint32_t n, uint32_t *out)
{
	if (!out && n) return PP_INVALID_ARGS;
	DevBuf d;
	PP_CK(d.alloc((size_t) n * 16));
	PP_CK(launch_philox_fill(c0, c1, c2, c3, k0, k1, n, d.as<uint32_t>(), 0));
	PP_CK(cudaMemcpy(out, d.p, (size_t) n * 16, cudaMemcpyDeviceToHost));
	return PP_SUCCESS;
}

extern "C" int pp_move_host(const PPParameters *params, uint64_t seed,
	uint32_t iter, uint32_t n, const uint32_t *cell_in, const uint32_t *en_in,
	uint32_t *cell_out, uint32_t *en_out)
{
	if (!params) return PP_INVALID_ARGS;
	RunSpec s{};
	s.p = *params;
	s.seed = seed;
	s.iters = 0xffffffffu;
	RunDev run = make_run(s, 0, 1, 0, 0, 0);
	DevBuf ki, vi, ko, vo, rd;
	size_t b = (size_t) n * 4;
	PP_CK(ki.alloc(b)); PP_CK(vi.alloc(b)); PP_CK(ko.alloc(b)); PP_CK(vo.alloc(b));
	PP_CK(rd.alloc(sizeof(RunDev)));
	PP_CK(cudaMemcpy(ki.p, cell_in, b, cudaMemcpyHostToDevice));
	PP_CK(cudaMemcpy(vi.p, en_in, b, cudaMemcpyHostToDevice));
	PP_CK(cudaMemcpy(rd.p, &run, sizeof(RunDev), cudaMemcpyHostToDevice));
	PP_CK(launch_move_only(ki.as<uint32_t>(), vi.as<uint32_t>(),
		ko.as<uint32_t>(), vo.as<uint32_t>(), n, rd.as<RunDev>(), iter,
		params->grid_x * params->grid_y, 0));
	PP_CK(cudaMemcpy(cell_out, ko.p, b, cudaMemcpyDeviceToHost));
	PP_CK(cudaMemcpy(en_out, vo.p, b, cudaMemcpyDeviceToHost));
	return PP_SUCCESS;
}

extern "C" int pp_lookback_selftest(uint32_t n_chunks, int32_t stall_chunk,
	uint32_t *prefix_out)
{
	if (n_chunks == 0 || n_chunks > 4096) return PP_INVALID_ARGS;
	DevBuf lb, misc, pre;
	PP_CK(lb.alloc((size_t) n_chunks * 8));
	PP_CK(misc.alloc(8));
	PP_CK(pre.alloc((size_t) n_chunks * 4));
	PP_CK(cudaMemset(lb.p, 0, (size_t) n_chunks * 8));
	PP_CK(cudaMemset(misc.p, 0, 8));
	PP_CK(cudaMemset(pre.p, 0, (size_t) n_chunks * 4));
	uint32_t *ticket = misc.as<uint32_t>(), *err = ticket + 1;
	/* about 2^14 polls (tens of milliseconds) before a wait gives up */
	PP_CK(launch_lookback_selftest(lb.as<uint64_t>(), ticket, err,
		pre.as<uint32_t>(), n_chunks,
		stall_chunk < 0 ? 0xffffffffu : (uint32_t) stall_chunk, 1u << 14, 0));
	PP_CK(cudaDeviceSynchronize());
	uint32_t e = 0;
	PP_CK(cudaMemcpy(&e, err, 4, cudaMemcpyDeviceToHost));
	if (prefix_out)
		PP_CK(cudaMemcpy(prefix_out, pre.p, (size_t) n_chunks * 4, cudaMemcpyDeviceToHost));
	return (e & ERRF_TIMEOUT) ? PP_ERR_TIMEOUT : PP_SUCCESS;
}

extern "C" int pp_radix_sort_host(uint32_t n, const uint32_t *keys_in,
	const uint32_t *vals_in, uint32_t *keys_out, uint32_t *vals_out,
	uint32_t key_bits, uint32_t digit_bits)
{
	if (key_bits == 0 || key_bits > 32) return PP_INVALID_ARGS;
	uint32_t d = digit_bits;
	if (d == 0) {
		uint32_t passes = (key_bits + 7) / 8;
		d = (key_bits + passes - 1) / passes;
		if (d < 5) d = 5;
	}
	if (d < 5 || d > 8) return PP_INVALID_ARGS;
	uint32_t passes = (key_bits + d - 1) / d;
	int sms = 0;
	PP_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
	size_t b = (size_t) n * 4;
	size_t tiles = ceil_div(n, SORT_TILE) + 1;
	DevBuf k0, v0, k1, v1, lb, ctr, hist, nd;
	PP_CK(k0.alloc(b)); PP_CK(v0.alloc(b)); PP_CK(k1.alloc(b)); PP_CK(v1.alloc(b));
	PP_CK(lb.alloc(tiles * 256 * 8));
	PP_CK(ctr.alloc(sizeof(WorldCounters)));
	PP_CK(hist.alloc(8 * 256 * 4));
	PP_CK(nd.alloc(4));
	PP_CK(cudaMemset(lb.p, 0, tiles * 256 * 8));
	PP_CK(cudaMemset(ctr.p, 0, sizeof(WorldCounters)));
	PP_CK(cudaMemset(hist.p, 0, 8 * 256 * 4));
	PP_CK(cudaMemcpy(nd.p, &n, 4, cudaMemcpyHostToDevice));
	PP_CK(cudaMemcpy(k0.p, keys_in, b, cudaMemcpyHostToDevice));
	PP_CK(cudaMemcpy(v0.p, vals_in, b, cudaMemcpyHostToDevice));
	PP_CK(launch_radix_hist(k0.as<uint32_t>(), nd.as<uint32_t>(),
		hist.as<uint32_t>(), d, passes, sms * 4, 0));
	uint32_t *ki = k0.as<uint32_t>(), *vi = v0.as<uint32_t>();
	uint32_t *ko = k1.as<uint32_t>(), *vo = v1.as<uint32_t>();
	int occ = occupancy_sort((int) d);
	for (uint32_t p = 0; p < passes; p++) {
		PP_CK(launch_radix_pass(ki, vi, ko, vo, hist.as<uint32_t>() + p * 256,
			lb.as<uint64_t>(), ctr.as<WorldCounters>(), nd.as<uint32_t>(), p,
			p * d, d, sms * (occ > 0 ? occ : 1), 0));
		std::swap(ki, ko);
		std::swap(vi, vo);
	}
	PP_CK(cudaDeviceSynchronize());
	WorldCounters c{};
	PP_CK(cudaMemcpy(&c, ctr.p, sizeof(c), cudaMemcpyDeviceToHost));
	if (c.err & ERRF_TIMEOUT) return PP_ERR_TIMEOUT;
	PP_CK(cudaMemcpy(keys_out, ki, b, cudaMemcpyDeviceToHost));
	PP_CK(cudaMemcpy(vals_out, vi, b, cudaMemcpyDeviceToHost));
	return PP_SUCCESS;
}

extern "C" int pp_cell_offsets_host(uint32_t n, const uint32_t *sorted_keys,
	uint32_t n_cells, uint32_t *off)
{
	int sms = 0;
	PP_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
	DevBuf k, o, nd;
	PP_CK(k.alloc((size_t) n * 4));
	PP_CK(o.alloc(((size_t) n_cells + 1) * 4));
	PP_CK(nd.alloc(4));
	PP_CK(cudaMemcpy(k.p, sorted_keys, (size_t) n * 4, cudaMemcpyHostToDevice));
	PP_CK(cudaMemcpy(nd.p, &n, 4, cudaMemcpyHostToDevice));
	PP_CK(launch_offsets(k.as<uint32_t>(), nd.as<uint32_t>(), 0, n_cells,
		o.as<uint32_t>(), sms * 8, 0));
	PP_CK(cudaMemcpy(off, o.p, ((size_t) n_cells + 1) * 4, cudaMemcpyDeviceToHost));
	return PP_SUCCESS;
}

/* ---------------- batched runs ---------------- */

extern "C" void pp_batch_opts_default(pp_batch_opts *o)
{
	memset(o, 0, sizeof(*o));
	o->pool_factor = 4;
	o->use_graph = 1;
	o->stats_chunk = 1024;
}

extern "C" int pp_batch_autotune(const pp_run_desc *runs, int n_runs,
	const pp_batch_opts *opts, pp_tuning *out)
{
	/* tune on the run with the most cells, at the batch's pool density */
	if (!runs || n_runs <= 0 || !out) return PP_INVALID_ARGS;
	pp_batch_opts o;
	if (opts) o = *opts;
	else pp_batch_opts_default(&o);
	uint64_t n0 = 0, cells = 0;
	int big = 0;
	for (int r = 0; r < n_runs; r++) {
		const PPParameters &p = runs[r].params;
		n0 += (uint64_t) p.init_sheep + p.init_wolves;
		cells += (uint64_t) p.grid_x * p.grid_y;
		if ((uint64_t) p.grid_x * p.grid_y
			> (uint64_t) runs[big].params.grid_x * runs[big].params.grid_y) big = r;
	}
	const uint32_t pf = o.pool_factor ? o.pool_factor : 4;
	const uint64_t cap = std::min<uint64_t>(std::max<uint64_t>(pf * n0, 1024), 0x7fffffffu);
	PPParameters bp = runs[big].params;
	bp.grid_xy = bp.grid_x * bp.grid_y;
	const uint32_t bcap = (uint32_t) std::min<uint64_t>(0x7fffffffu,
		(uint64_t) ((double) cap * bp.grid_xy / std::max<uint64_t>(cells, 1)) + 1024);
	return pp_autotune(&bp, runs[big].seed, bcap, o.device, out);
}

extern "C" int pp_batch_run(const pp_run_desc *runs, int n_runs,
	const pp_batch_opts *opts, pp_stats_cb cb, void *user)
{
	pp::NvtxRange nvtx_range("pp_batch_run");
	if (!runs || n_runs <= 0) return PP_INVALID_ARGS;
	pp_batch_opts o;
	if (opts) o = *opts;
	else pp_batch_opts_default(&o);
	std::vector<RunSpec> specs(n_runs);
	uint64_t n0 = 0, cells = 0;
	uint32_t max_iters = 0;
	for (int r = 0; r < n_runs; r++) {
		PPParameters p = runs[r].params;
		p.grid_xy = p.grid_x * p.grid_y;
		int rc = pp_params_check(&p, nullptr, 0);
		if (rc) return rc;
		specs[r].p = p;
		specs[r].seed = runs[r].seed;
		specs[r].iters = p.iters;
		rc = agent_energy_bits(o.agent_size, p, &specs[r].energy_bits);
		if (rc) return rc;
		n0 += (uint64_t) p.init_sheep + p.init_wolves;
		cells += p.grid_xy;
		max_iters = std::max(max_iters, p.iters);
	}
	WorldConfig cfg;
	cfg.device = o.device;
	uint32_t pf = o.pool_factor ? o.pool_factor : 4;
	cfg.cap = (uint32_t) std::min<uint64_t>(std::max<uint64_t>(pf * n0, 1024), 0x7fffffffu);
	cfg.tile_cells = o.tile_cells;
	cfg.digit_bits = o.sort_digit_bits;
	cfg.graph_iters = o.use_graph ? 32 : 0;
	if (o.autotune && o.tile_cells == 0) {
		pp_tuning tu;
		int trc = pp_batch_autotune(runs, n_runs, &o, &tu);
		if (trc) return trc;
		cfg.tile_cells = tu.tile_cells;
		cfg.fused = tu.sort_pipeline == 0;
		if (tu.sort_digit_bits) cfg.digit_bits = tu.sort_digit_bits;
	}
	uint32_t chunk = o.stats_chunk ? o.stats_chunk : 1024;
	cfg.ring_rows = std::max<uint32_t>(chunk + 1, 64);
	World w;
	int rc = w.create(specs, cfg);
	if (rc) return rc;
	std::vector<std::vector<PPStatistics>> rows(n_runs);
	for (int r = 0; r < n_runs; r++) {
		rows[r].resize((size_t) specs[r].iters + 1);
		rc = w.read_rows((uint32_t) r, 0, 0, rows[r].data());
		if (rc) return rc;
	}
	uint32_t g = 0;
	while (g < max_iters) {
		uint32_t c = std::min(max_iters - g, chunk);
		rc = w.enqueue(c);
		if (rc) return rc;
		rc = w.sync_check();
		if (rc) return rc;
		for (int r = 0; r < n_runs; r++) {
			uint32_t it = specs[r].iters;
			if (g >= it) continue;
			uint32_t hi = std::min(g + c, it);
			rc = w.read_rows((uint32_t) r, g + 1, hi, rows[r].data() + g + 1);
			if (rc) return rc;
			if (hi == it && cb) cb(r, rows[r].data(), it + 1, user);
		}
		g += c;
	}
	if (max_iters == 0 && cb)
		for (int r = 0; r < n_runs; r++) cb(r, rows[r].data(), 1, user);
	return PP_SUCCESS;
}
