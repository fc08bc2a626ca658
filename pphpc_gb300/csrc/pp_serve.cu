/*
 * pp_serve.cu -- continuous batching of simulation requests.
 *
 * The reference runs one simulation per process (opencl/pp/pp_gpu.c:1700).
 * A server here owns one world whose tile space and agent pool are sized
 * from a device-memory budget. Submitted runs wait in a FIFO queue; at each
 * poll the queue head is admitted while a run slot, a contiguous tile range
 * and its agent-pool reservation are free, then every resident run advances
 * through the same launches (their work shares every kernel), the new
 * stats rows of each resident run are streamed to the host, and finished
 * runs release their slot, tiles and reservation. A run's draws are keyed
 * by its own seed, its own iteration and its own slot ids, so its stats are
 * identical alone and in any mix.
 */
#include <algorithm>
#include <deque>
#include <map>
#include <new>

#include "pp_world.cuh"

using namespace pp;

extern "C" int pp_params_check(const PPParameters *p, char *errmsg, size_t errlen);

namespace {

struct Request {
	uint64_t id = 0;
	RunSpec spec;
	int status = PP_SUCCESS;
	uint32_t slot = 0;
	bool resident = false, done = false;
	uint32_t start_g = 0;
	uint32_t n_rows = 0;          /* rows available */
	uint64_t reserve = 0;
	std::vector<PPStatistics> rows;
	bool has_focal = false;
	pp_focal focal;
};

uint64_t reservation(const RunSpec &s, uint32_t pool_factor)
{
	uint64_t n0 = (uint64_t) s.p.init_sheep + s.p.init_wolves;
	uint64_t cells = (uint64_t) s.p.grid_x * s.p.grid_y;
	/* Populations of the v2 parameter set reach ~2.2 agents per cell. */
	return std::max<uint64_t>(pool_factor * n0, (cells * 5) / 2) + 64;
}

} /* namespace */

struct pp_server {
	World world;
	pp_serve_opts opts;
	std::deque<uint64_t> queue;
	std::deque<uint64_t> finished;      /* done, not yet listed by pp_serve_finished */
	/* pinned host copy of the stats ring rows one poll produced, every
	 * slot up to the highest resident one */
	PPStatistics *ring_host = nullptr;
	~pp_server() { if (ring_host) cudaFreeHost(ring_host); }
	std::map<uint64_t, Request> reqs;
	std::vector<uint64_t> slot_req;
	uint64_t next_id = 1;
	uint64_t reserved = 0;
	uint32_t cap = 0;
	uint32_t max_tiles = 0;
	int fatal = PP_SUCCESS;
};

extern "C" void pp_serve_opts_default(pp_serve_opts *o)
{
	memset(o, 0, sizeof(*o));
	o->device = 0;
	o->mem_budget_bytes = 8ull << 30;
	o->max_runs = 256;
	o->pool_factor = 4;
	o->stats_chunk = 64;
	o->ss_from = 1000;
}

extern "C" int pp_serve_create(const pp_serve_opts *opts, pp_server **out)
{
	if (!out) return PP_INVALID_ARGS;
	*out = nullptr;
	pp_serve_opts o;
	if (opts) o = *opts;
	else pp_serve_opts_default(&o);
	if (o.max_runs == 0 || o.max_runs > 60000) return PP_INVALID_ARGS;
	if (o.tile_cells != 0 && o.tile_cells != 512 && o.tile_cells != 1024
		&& o.tile_cells != 2048) return PP_INVALID_ARGS;
	if (o.agent_size != 0 && o.agent_size != 32 && o.agent_size != 64)
		return PP_INVALID_ARGS;
	pp_server *srv = new (std::nothrow) pp_server();
	if (!srv) return PP_OUT_OF_RESOURCES;
	srv->opts = o;
	/* Budget split: a tile costs 2 B per cell (grass) plus ~610 B of
	 * per-tile tables (inboxes, offsets, partial stats), an agent slot 101 B
	 * (a new run's agents in creation order and bucketed by tile, 24 B; two
	 * group buffers of three slots per agent; seven scratch words for
	 * crowded tiles; sort look-back). Cells are bounded by the 2^31 key space. */
	/* 2048-cell tiles by default: on a 1000-request stream of 100^2 to
	 * 3200^2 runs they served 2.17e10 agent-steps/s against 1.86e10 on
	 * 1024-cell tiles and 2.01e10 on 512 */
	const uint32_t T = o.tile_cells ? o.tile_cells : 2048;
	const uint64_t tile_bytes = T * 2ull + 610;
	uint64_t budget = o.mem_budget_bytes;
	uint64_t cell_bytes = budget / 8;
	uint64_t tiles = cell_bytes / tile_bytes;
	uint64_t max_tiles = ((1ull << 31) / T) - 1;
	if (tiles > max_tiles) tiles = max_tiles;
	if (tiles < 1) tiles = 1;
	uint64_t rest = budget > tiles * tile_bytes ? budget - tiles * tile_bytes : 0;
	uint64_t cap = rest / 101;
	if (cap > 0x7fffffffull) cap = 0x7fffffffull;
	if (cap < 4096) cap = 4096;
	WorldConfig cfg;
	cfg.device = o.device;
	cfg.tile_cells = T;
	cfg.cap = (uint32_t) cap;
	cfg.extra_tiles = (uint32_t) tiles;
	cfg.nruns_cap = o.max_runs;
	cfg.ring_rows = std::max<uint32_t>(o.stats_chunk + 1, 64);
	cfg.graph_iters = 0;
	/* Dense v2 runs put up to ~2.2 agents per cell in a tile; tiles above
	 * the shared-memory capacity take the act's crowded path. */
	cfg.act_cap = std::min<uint32_t>(2 * T, 2048);
	std::vector<RunSpec> none;
	int rc = srv->world.create(none, cfg);
	if (rc) {
		delete srv;
		cudaGetLastError();
		return rc;
	}
	if (cudaMallocHost(&srv->ring_host, (size_t) cfg.ring_rows * o.max_runs
			* sizeof(PPStatistics)) != cudaSuccess) {
		cudaGetLastError();
		srv->ring_host = nullptr;
		delete srv;
		return PP_OUT_OF_RESOURCES;
	}
	srv->cap = (uint32_t) cap;
	srv->max_tiles = (uint32_t) tiles;
	srv->slot_req.assign(o.max_runs, 0);
	*out = srv;
	return PP_SUCCESS;
}

extern "C" int pp_serve_submit(pp_server *srv, const pp_run_desc *run,
	uint64_t *id)
{
	if (!srv || !run) return PP_INVALID_ARGS;
	PPParameters p = run->params;
	p.grid_xy = p.grid_x * p.grid_y;
	int rc = pp_params_check(&p, nullptr, 0);
	if (rc) return rc;
	Request rq;
	rq.spec.p = p;
	rq.spec.seed = run->seed;
	rq.spec.iters = p.iters;
	rq.spec.ss_from = srv->opts.ss_from;
	rc = agent_energy_bits(srv->opts.agent_size, p, &rq.spec.energy_bits);
	if (rc) return rc;
	rq.reserve = reservation(rq.spec, srv->opts.pool_factor ? srv->opts.pool_factor : 4);
	const uint64_t T = srv->world.tile_cells();
	uint64_t tiles_needed = ((uint64_t) p.grid_xy + T - 1) / T;
	if (rq.reserve > srv->cap || tiles_needed > srv->max_tiles)
		return PP_OUT_OF_RESOURCES; /* can never be admitted */
	rq.rows.resize((size_t) p.iters + 1);
	uint64_t rid = srv->next_id++;
	rq.id = rid;
	srv->reqs.emplace(rid, std::move(rq));
	srv->queue.push_back(rid);
	if (id) *id = rid;
	return PP_SUCCESS;
}

static int finish_request(pp_server *srv, Request &rq, int status)
{
	int rc = PP_SUCCESS;
	if (rq.resident && status == PP_SUCCESS) {
		FocalDev f;
		rc = srv->world.read_focal(rq.slot, &f);
		if (rc == PP_SUCCESS) {
			focal_export(f, &rq.focal);
			rq.has_focal = true;
		}
	}
	if (rq.resident) {
		rc = srv->world.retire(rq.slot);
		srv->slot_req[rq.slot] = 0;
		srv->reserved -= rq.reserve;
		rq.resident = false;
	}
	rq.done = true;
	rq.status = status;
	srv->finished.push_back(rq.id);
	return rc;
}

extern "C" int pp_serve_cancel(pp_server *srv, uint64_t id)
{
	if (!srv) return PP_INVALID_ARGS;
	auto it = srv->reqs.find(id);
	if (it == srv->reqs.end()) return PP_INVALID_ARGS;
	Request &rq = it->second;
	if (rq.done) return PP_SUCCESS;
	auto q = std::find(srv->queue.begin(), srv->queue.end(), id);
	if (q != srv->queue.end()) srv->queue.erase(q);
	return finish_request(srv, rq, PP_ERR_CANCELLED);
}

static int admit_queued(pp_server *srv)
{
	World &w = srv->world;
	while (!srv->queue.empty()) {
		uint64_t id = srv->queue.front();
		Request &rq = srv->reqs[id];
		if (srv->reserved + rq.reserve > srv->cap || !w.fits(rq.spec)) break;
		uint32_t slot = 0;
		int rc = w.admit(rq.spec, &slot);
		if (rc == PP_OUT_OF_RESOURCES) break;
		if (rc) return rc;
		srv->queue.pop_front();
		rq.resident = true;
		rq.slot = slot;
		rq.start_g = w.giter();
		srv->slot_req[slot] = id;
		srv->reserved += rq.reserve;
		rc = w.read_rows(slot, rq.start_g, rq.start_g, rq.rows.data());
		if (rc) return rc;
		rq.n_rows = 1;
		if (rq.spec.iters == 0) finish_request(srv, rq, PP_SUCCESS);
	}
	return PP_SUCCESS;
}

extern "C" int pp_serve_poll(pp_server *srv, uint32_t n_iters)
{
	pp::NvtxRange nvtx_range("pp_serve_poll");
	if (!srv) return PP_INVALID_ARGS;
	if (srv->fatal) return srv->fatal;
	World &w = srv->world;
	int rc = admit_queued(srv);
	if (rc) return srv->fatal = rc;
	bool any = false;
	for (uint64_t id : srv->slot_req) if (id) { any = true; break; }
	if (!any || n_iters == 0) return PP_SUCCESS;
	uint32_t steps = std::min<uint32_t>(n_iters, w.ring_rows() - 1);
	uint32_t g0 = w.giter();
	rc = w.enqueue(steps);
	if (rc == PP_SUCCESS) rc = w.sync_check();
	if (rc) {
		for (uint64_t id : srv->slot_req)
			if (id) finish_request(srv, srv->reqs[id], rc);
		return srv->fatal = rc;
	}
	uint32_t g1 = g0 + steps;
	/* rows g0 + 1 .. g1 of every slot up to the highest resident one, in
	 * one copy (a resident run has read every row up to g0) */
	uint32_t nslots = 0;
	for (uint32_t s = 0; s < srv->slot_req.size(); s++)
		if (srv->slot_req[s]) nslots = s + 1;
	rc = w.read_ring(g0 + 1, g1, nslots, srv->ring_host);
	if (rc) return srv->fatal = rc;
	for (uint32_t s = 0; s < nslots; s++) {
		uint64_t id = srv->slot_req[s];
		if (!id) continue;
		Request &rq = srv->reqs[id];
		uint32_t last = rq.start_g + rq.spec.iters;
		uint32_t lo = rq.start_g + rq.n_rows;
		uint32_t hi = std::min(g1, last);
		for (uint32_t g = lo; g <= hi; g++)
			rq.rows[g - rq.start_g] = srv->ring_host[(size_t) (g - g0 - 1) * nslots + s];
		if (hi >= lo) rq.n_rows = hi - rq.start_g + 1;
		if (hi == last) finish_request(srv, rq, PP_SUCCESS);
	}
	return PP_SUCCESS;
}

extern "C" int pp_serve_read(pp_server *srv, uint64_t id, uint32_t first,
	uint32_t n, PPStatistics *rows, uint32_t *n_out)
{
	if (!srv) return PP_INVALID_ARGS;
	auto it = srv->reqs.find(id);
	if (it == srv->reqs.end()) return PP_INVALID_ARGS;
	Request &rq = it->second;
	uint32_t avail = rq.n_rows > first ? rq.n_rows - first : 0;
	uint32_t m = std::min(avail, n);
	if (m && rows) memcpy(rows, rq.rows.data() + first, (size_t) m * sizeof(PPStatistics));
	if (n_out) *n_out = m;
	return PP_SUCCESS;
}

extern "C" int pp_serve_focal(pp_server *srv, uint64_t id, pp_focal *out)
{
	if (!srv || !out) return PP_INVALID_ARGS;
	auto it = srv->reqs.find(id);
	if (it == srv->reqs.end() || !it->second.has_focal) return PP_INVALID_ARGS;
	*out = it->second.focal;
	return PP_SUCCESS;
}

extern "C" int pp_serve_status(pp_server *srv, uint64_t id, pp_serve_event *ev)
{
	if (!srv || !ev) return PP_INVALID_ARGS;
	auto it = srv->reqs.find(id);
	if (it == srv->reqs.end()) return PP_INVALID_ARGS;
	Request &rq = it->second;
	ev->id = id;
	ev->status = rq.status;
	ev->n_rows = rq.n_rows;
	ev->done = rq.done ? 1 : 0;
	return PP_SUCCESS;
}

extern "C" int pp_serve_finished(pp_server *srv, uint64_t *ids, uint32_t max,
	uint32_t *n_out)
{
	if (!srv || !n_out || (max && !ids)) return PP_INVALID_ARGS;
	uint32_t n = 0;
	while (n < max && !srv->finished.empty()) {
		ids[n++] = srv->finished.front();
		srv->finished.pop_front();
	}
	*n_out = n;
	return PP_SUCCESS;
}

extern "C" int pp_serve_load(pp_server *srv, uint32_t *queued, uint32_t *resident)
{
	if (!srv) return PP_INVALID_ARGS;
	if (queued) *queued = (uint32_t) srv->queue.size();
	uint32_t r = 0;
	for (uint64_t id : srv->slot_req) if (id) r++;
	if (resident) *resident = r;
	return PP_SUCCESS;
}

extern "C" int pp_serve_release(pp_server *srv, uint64_t id)
{
	if (!srv) return PP_INVALID_ARGS;
	auto it = srv->reqs.find(id);
	if (it == srv->reqs.end()) return PP_INVALID_ARGS;
	if (!it->second.done) return PP_INVALID_ARGS;
	srv->reqs.erase(it);
	return PP_SUCCESS;
}

extern "C" int pp_serve_destroy(pp_server *srv)
{
	delete srv;
	return PP_SUCCESS;
}
