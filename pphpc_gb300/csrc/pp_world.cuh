/*
 * pp_world.cuh -- host-side owner of one world: device buffers, the run
 * table, the per-iteration launch sequence (captured as CUDA graphs) and
 * the stats ring. A single simulation is a world of one run; batched and
 * served runs share one world.
 */
#pragma once

#include <utility>
#include <vector>
#include <cstring>

#include <nvtx3/nvToolsExt.h>

#include "pp_kernels.cuh"

namespace pp {

/* A named NVTX range over a host-side phase (create, step, admission, poll,
 * tuning), for timeline tools; without one attached it costs nothing. */
struct NvtxRange {
	explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
	~NvtxRange() { nvtxRangePop(); }
	NvtxRange(const NvtxRange &) = delete;
	NvtxRange &operator=(const NvtxRange &) = delete;
};

struct RunSpec {
	PPParameters p;
	uint64_t seed;
	uint32_t iters;          /* UINT32_MAX = open-ended */
	/* A run resumed from a snapshot (host arrays, run-local cells in
	 * canonical order, grass countdowns) at iteration start_iter; null
	 * init_val = a fresh run initialised from its seed. */
	const uint32_t *init_cell = nullptr, *init_val = nullptr;
	const uint16_t *init_grass = nullptr;
	uint32_t init_n = 0;
	uint32_t start_iter = 0;
	uint32_t ss_from = 1000;  /* focal measures: steady state is t > ss_from */
	uint32_t energy_bits = 30; /* energy field width (11, 16 or 30)        */
	uint64_t agents() const
	{
		return init_val ? (uint64_t) init_n : (uint64_t) p.init_sheep + p.init_wolves;
	}
};

/* Device buffers through the process-wide cache (pp_alloc.cu): *got is
 * the size of the buffer handed out (at least bytes), to be passed back to
 * cached_free. */
cudaError_t cached_malloc(int device, size_t bytes, void **p, size_t *got);
void cached_free(int device, void *p, size_t bytes);

/* Energy field width for the reference's agent size (0, 32 or 64) on a
 * grid of p (32-bit agents hold 10-bit coordinates, pp_gpu.cl:236-316). */
int agent_energy_bits(uint32_t agent_size, const PPParameters &p, uint32_t *bits);

struct WorldConfig {
	int device = 0;
	uint32_t tile_cells = 0;       /* 0 = choose */
	uint32_t digit_bits = 0;       /* 0 = choose */
	uint32_t cap = 0;              /* agent slots */
	uint32_t ring_rows = 4096;
	uint32_t graph_iters = 32;     /* iterations per captured graph, 0 = no graphs */
	uint32_t nruns_cap = 0;        /* run slots (>= number of runs) */
	uint32_t extra_tiles = 0;      /* free tile space for later admissions */
	uint32_t act_cap = 0;          /* 0 = choose */
	uint32_t max_cells_hint = 0;   /* largest run (cells), for serving worlds */
	bool fused = true;             /* fused act+move iteration (else the sort pipeline) */
};

class World {
public:
	World() {}
	~World();

	/* Build the world for the given runs (each initialised at world
	 * iteration 0). Returns a pp_error_codes value. */
	int create(const std::vector<RunSpec> &runs, const WorldConfig &cfg);

	/* Enqueue n iterations; no host synchronisation. */
	int enqueue(uint32_t n);
	/* capture the iteration graph now if a call of n iterations would, so
	 * that a timed call does not include the capture */
	int prepare_graph(uint32_t n);

	/* Wait and check the device error flags. */
	int sync_check();

	/* Copy the stats rows of run r for world iterations [g0, g1] (ring
	 * positions must still be valid). */
	int read_rows(uint32_t r, uint32_t g0, uint32_t g1, PPStatistics *out);
	/* Rows of world iterations [g0, g1] of run slots [0, nslots), row by
	 * row (out[(g - g0) * nslots + r]), in one copy per contiguous part of
	 * the ring. */
	int read_ring(uint32_t g0, uint32_t g1, uint32_t nslots, PPStatistics *out);

	/* Admission of a run into a free slot and tile range (serving). */
	int admit(const RunSpec &spec, uint32_t *slot_out);
	int retire(uint32_t slot);
	/* The running focal measures of run slot r (synchronises). */
	int read_focal(uint32_t r, FocalDev *out);
	bool fits(const RunSpec &spec) const;

	uint32_t giter() const { return giter_; }
	uint32_t nruns() const { return (uint32_t) runs_h_.size(); }
	const RunDev &run(uint32_t r) const { return runs_h_[r]; }
	uint32_t n_agents_dev();      /* reads the device counter (syncs) */
	cudaStream_t stream() const { return s_; }
	int dev_index() const { return device_; }
	WorldDev &dev() { return w_; }
	const LaunchCfg &launch() const { return lc_; }
	size_t bytes() const { return bytes_; }
	uint32_t ring_rows() const { return w_.ring_rows; }
	uint32_t tile_cells() const { return 1u << w_.log_tile; }
	bool fused() const { return w_.fused != 0; }
	int get_state(uint32_t *cell, uint32_t *en, uint32_t n_max,
		uint32_t *n_out, uint16_t *grass, uint32_t r);

	/* Run n iterations without graphs, timing every kernel with CUDA
	 * events on the world's stream; fills prof[0..4] (move, radix pass,
	 * offsets, act, finish) with algorithmic bytes (the fused pipeline
	 * launches only act and finish). */
	int profile(uint32_t n, pp_kernel_prof *prof, double *agent_steps);

private:
	int alloc(size_t bytes, void **p);
	int sort_into(uint32_t n, uint32_t *dst_k, uint32_t *dst_v);
	int load_run_state(const RunSpec &spec, const RunDev &run, uint32_t base,
		PPStatistics *row0);
	int build_graph();
	void drop_graph();
	int init_run_device(uint32_t r, uint32_t base, const RunSpec &spec);
	cudaError_t enqueue_one(const cudaEvent_t *marks = nullptr);
	int get_state_fused(uint32_t *cell, uint32_t *en, uint32_t n_max,
		uint32_t *n_out, uint32_t r);
	int place_bucketed(uint32_t n, uint32_t first, uint32_t count,
		uint32_t out_base);
	void free_all();

	int device_ = 0;
	cudaStream_t s_ = nullptr;
	WorldDev w_{};
	LaunchCfg lc_{};
	std::vector<RunDev> runs_h_;
	std::vector<uint16_t> tile_run_h_;
	std::vector<std::pair<void *, size_t>> allocs_;
	size_t bytes_ = 0;
	uint32_t giter_ = 0;
	uint32_t graph_iters_ = 0;
	cudaGraphExec_t gexec_ = nullptr;
	cudaGraph_t graph_ = nullptr;
	uint32_t used_tiles_ = 0;
	uint32_t null_slot_ = 0;
	std::vector<std::pair<uint32_t, uint32_t>> free_tiles_; /* (first, count) */
	/* Tiles of retired runs, with the world iteration of retirement. */
	std::vector<std::pair<std::pair<uint32_t, uint32_t>, uint32_t>> pending_tiles_;
	void release_pending();
	int update_tile_hi();
	uint32_t tile_hi_ = 0;    /* mirror of ctr->tile_hi */
	uint32_t agents_reserved_ = 0;
	uint32_t adm_used_ = 0;   /* admission area of the region buffer in use */
	uint32_t fslot_base_ = 0; /* regrowth histograms of admitted runs start here */
	static constexpr uint32_t FSLOT = 32768;   /* histogram room per admitted run */
	static constexpr uint32_t REBASE = 8192;   /* iterations between re-basings */
public:
	uint64_t h2d_ = 0, d2h_ = 0;   /* bytes copied host<->device by the world */
private:
	std::vector<uint32_t> reserve_of_;
};

/* Mean and standard deviation from the running sums (C ABI form). */
void focal_export(const FocalDev &f, pp_focal *out);

/* Pick tile size and digit width for a world. */
void choose_geometry(uint32_t total_cells, uint32_t cap, WorldConfig &cfg);

int cuda_status(cudaError_t e);

} /* namespace pp */
