/*
 * pp_tune.cu -- autotuner of the launch geometry.
 *
 * The reference fixes its work sizes by hand or by command-line options
 * (opencl/pp/pp_gpu.c:310-410: the --l-* local work sizes, the sort
 * options). Here the geometry of a world -- the iteration pipeline (fused
 * act+move, or move + radix sort + act), the cells per tile (which sets the
 * cells handled per thread of the act and the CTAs in flight) and, for the
 * sort pipeline, the radix digit width -- is measured: every candidate runs
 * a sample of the workload (the same parameters on a grid of at most
 * 4096 x 4096 cells, agents scaled by area, so the density is the
 * workload's) past its first population swing, and the candidate with the
 * lowest device time per agent-step wins. Results are cached per device and
 * workload shape for the life of the process; PP_TUNE_CACHE names an
 * optional file that keeps them across processes.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "pp_world.cuh"

using namespace pp;

extern "C" int pp_params_check(const PPParameters *p, char *errmsg, size_t errlen);

namespace {

/* Workload shape: device, log2 of the sample's cells, the pool density in
 * eighths of an agent per cell, and every model parameter that changes the
 * population's course. */
using TuneKey = std::tuple<int, int, int, std::string>;

std::mutex g_mu;
std::map<TuneKey, pp_tuning> g_cache;
bool g_file_loaded = false;

std::string params_tag(const PPParameters &p)
{
	char b[160];
	snprintf(b, sizeof(b), "%u,%u,%u,%u,%u,%u,%u,%u,%u",
		p.sheep_gain_from_food, p.sheep_reproduce_threshold,
		p.sheep_reproduce_prob, p.wolves_gain_from_food,
		p.wolves_reproduce_threshold, p.wolves_reproduce_prob,
		p.grass_restart,
		(uint32_t) llround(1e6 * p.init_sheep / std::max(1.0, (double) p.grid_x * p.grid_y)),
		(uint32_t) llround(1e6 * p.init_wolves / std::max(1.0, (double) p.grid_x * p.grid_y)));
	return b;
}

void load_file_cache()
{
	if (g_file_loaded) return;
	g_file_loaded = true;
	const char *fn = getenv("PP_TUNE_CACHE");
	if (!fn) return;
	FILE *f = fopen(fn, "r");
	if (!f) return;
	int dev, lc, dens;
	char tag[160];
	unsigned tile, sortp, digits;
	float cost;
	while (fscanf(f, "%d %d %d %159s %u %u %u %f", &dev, &lc, &dens, tag, &tile,
		&sortp, &digits, &cost) == 8) {
		pp_tuning t{};
		t.tile_cells = tile;
		t.sort_pipeline = sortp;
		t.sort_digit_bits = digits;
		t.ns_per_agent_step = cost;
		g_cache[TuneKey(dev, lc, dens, tag)] = t;
	}
	fclose(f);
}

void save_file_cache(const TuneKey &k, const pp_tuning &t)
{
	const char *fn = getenv("PP_TUNE_CACHE");
	if (!fn) return;
	FILE *f = fopen(fn, "a");
	if (!f) return;
	fprintf(f, "%d %d %d %s %u %u %u %g\n", std::get<0>(k), std::get<1>(k),
		std::get<2>(k), std::get<3>(k).c_str(), t.tile_cells, t.sort_pipeline,
		t.sort_digit_bits, (double) t.ns_per_agent_step);
	fclose(f);
}

/* Device ns per agent-step of one candidate on the sample, or a negative
 * pp_error_codes value. */
double measure(const RunSpec &spec, uint32_t cap, int device, bool fused,
	uint32_t tile, uint32_t warm, uint32_t timed)
{
	World w;
	WorldConfig cfg;
	cfg.device = device;
	cfg.cap = cap;
	cfg.tile_cells = tile;
	cfg.fused = fused;
	cfg.graph_iters = 0;
	cfg.ring_rows = std::max<uint32_t>(warm + timed + 2, 64);
	std::vector<RunSpec> runs(1, spec);
	int rc = w.create(runs, cfg);
	if (rc) return rc;
	rc = w.enqueue(warm);
	if (rc == PP_SUCCESS) rc = w.sync_check();
	if (rc) return rc;
	cudaEvent_t a, b;
	if (cudaEventCreate(&a) != cudaSuccess) return PP_ERR_CUDA;
	if (cudaEventCreate(&b) != cudaSuccess) { cudaEventDestroy(a); return PP_ERR_CUDA; }
	cudaEventRecord(a, w.stream());
	rc = w.enqueue(timed);
	cudaEventRecord(b, w.stream());
	if (rc == PP_SUCCESS) rc = w.sync_check();
	float ms = 0;
	if (rc == PP_SUCCESS && cudaEventElapsedTime(&ms, a, b) != cudaSuccess) rc = PP_ERR_CUDA;
	cudaEventDestroy(a);
	cudaEventDestroy(b);
	if (rc) return rc;
	std::vector<PPStatistics> rows(timed);
	rc = w.read_rows(0, warm, warm + timed - 1, rows.data());
	if (rc) return rc;
	double steps = 0;
	for (const PPStatistics &r : rows) steps += (double) r.sheep + r.wolves;
	if (steps <= 0) steps = 1;
	return 1e6 * ms / steps;
}

} /* namespace */

extern "C" int pp_autotune(const PPParameters *params, uint64_t seed,
	uint32_t max_agents, int device, pp_tuning *out)
{
	pp::NvtxRange nvtx_range("pp_autotune");
	if (!params || !out) return PP_INVALID_ARGS;
	PPParameters p = *params;
	p.grid_xy = p.grid_x * p.grid_y;
	int rc = pp_params_check(&p, nullptr, 0);
	if (rc) return rc;
	const uint64_t cells = (uint64_t) p.grid_x * p.grid_y;
	const uint64_t n0 = (uint64_t) p.init_sheep + p.init_wolves;
	const uint64_t cap_full = max_agents ? max_agents
		: std::max<uint64_t>(std::max<uint64_t>(4 * n0, 1024), 16777216ull);
	/* the sample: the workload itself, or a 4096 x 4096 grid at its density */
	PPParameters q = p;
	double scale = 1.0;
	if (cells > 4096ull * 4096ull) {
		q.grid_x = q.grid_y = 4096;
		scale = (double) (4096ull * 4096ull) / (double) cells;
		q.init_sheep = (uint32_t) llround(p.init_sheep * scale);
		q.init_wolves = (uint32_t) llround(p.init_wolves * scale);
	}
	q.grid_xy = q.grid_x * q.grid_y;
	const uint64_t qcells = (uint64_t) q.grid_x * q.grid_y;
	const uint32_t cap = (uint32_t) std::min<uint64_t>(
		std::max<uint64_t>((uint64_t) llround(cap_full * scale), 1024), 0x7fffffffu);
	int lc = 0;
	while ((1ull << lc) < qcells) lc++;
	const int dens = (int) std::min<double>(1e6, 8.0 * cap / std::max<uint64_t>(qcells, 1));
	const TuneKey key(device, lc, dens, params_tag(p));
	{
		std::lock_guard<std::mutex> g(g_mu);
		load_file_cache();
		auto it = g_cache.find(key);
		if (it != g_cache.end()) {
			*out = it->second;
			return PP_SUCCESS;
		}
	}
	/* long enough to see the population's first swing (the v2 set peaks
	 * near iteration 70), bounded */
	const uint32_t warm = std::min<uint32_t>(std::max<uint32_t>(p.iters / 8, 3), 96);
	const uint32_t timed = 16;
	RunSpec spec;
	spec.p = q;
	spec.seed = seed;
	spec.iters = 0xffffffffu;
	const uint32_t tiles[5] = {512, 1024, 2048, 4096, 8192};
	pp_tuning best{};
	double best_cost = 1e300;
	int last_err = PP_SUCCESS;
	for (int fused = 1; fused >= 0; fused--) {
		for (uint32_t t : tiles) {
			if (t > 4 * qcells && t != 1024) continue;   /* tiles far larger than the grid */
			if (t < 1024 && !fused) continue;            /* the sort pipeline's act needs 1024+ */
			double c = measure(spec, cap, device, fused != 0, t, warm, timed);
			if (c < 0) {
				last_err = (int) c;
				cudaGetLastError();
				continue;
			}
			if (c < best_cost) {
				best_cost = c;
				best.tile_cells = t;
				best.sort_pipeline = fused ? 0 : 1;
				best.sort_digit_bits = 0;
				best.ns_per_agent_step = (float) c;
			}
		}
	}
	if (best_cost >= 1e300) return last_err ? last_err : PP_LIBRARY_ERROR;
	{
		std::lock_guard<std::mutex> g(g_mu);
		g_cache[key] = best;
		save_file_cache(key, best);
	}
	*out = best;
	return PP_SUCCESS;
}
