/*
 * pp_cpu_host.cpp -- runs the reference's CPU kernels (pp_cpu_kernels.cpp,
 * the unmodified opencl/pp/pp_cpu.cl) the way the reference's host program
 * does, with host threads in place of an OpenCL CPU device.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle/ref/build_ref.py): the statistical
 * target of the parity tests and the timed CPU baseline. Nothing in the
 * product links it.
 *
 * Followed from opencl/pp/pp_cpu.c:
 *   work sizes       ppc_worksizes_calc, 232-325 (no -g/-l options: the
 *                    global work size is the maximum, rows / 3, and rows
 *                    per work item rows / gws, plus one when the remainder
 *                    allows it)
 *   initial check    main, 925-929 (initial agents must fit in max agents)
 *   buffers          ppc_datasizes_get 470-482, ppc_buffers_init 497-567
 *                    (every buffer filled with zeros)
 *   seeds            one RNG state per work item from the run seed
 *                    (clo_rng_new(..., CLO_RNG_SEED_HOST_MT, gws, seed),
 *                    931-933; SplitMix64 here, see ocl_compat.hpp)
 *   loop             ppc_simulate, 577-692: init over gws work items; per
 *                    iteration, rows_per_workitem launches of step1 (turn
 *                    t) and then rows_per_workitem launches of step2
 *                    (iteration, turn t)
 * A launch runs its work items on the host threads (OpenMP). Work items of
 * one launch touch rows at least three apart (pp_cpu.c:239-243), and each
 * draws only from its own RNG state, so the stats do not depend on the
 * thread count or schedule; the only shared writes are the slot
 * allocation (atomic compare-and-swap) and the stats (atomic adds), as in
 * the reference.
 */
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <omp.h>

namespace ocl {
thread_local unsigned long tl_gid, tl_gws;
unsigned max_agents, rows_per_workitem;
unsigned init_sheep, sheep_gain, sheep_thr, sheep_prob;
unsigned init_wolves, wolves_gain, wolves_thr, wolves_prob;
unsigned grass_restart, grid_x, grid_y, iters;
} /* namespace ocl */

extern "C" {
void ppr_kernel_init(void *agents, void *cells, void *stats, void *seeds,
	unsigned long gid, unsigned long gws);
void ppr_kernel_step1(void *agents, void *cells, void *seeds, unsigned turn,
	unsigned long gid, unsigned long gws);
void ppr_kernel_step2(void *agents, void *cells, void *seeds, void *stats,
	unsigned iter, unsigned turn, unsigned long gid, unsigned long gws);
unsigned long ppr_sizeof_agent(void);
unsigned long ppr_sizeof_cell(void);
unsigned long ppr_sizeof_stats(void);
}

namespace {

/* Minimum distance between the rows of one launch (PPC_D_MIN,
 * pp_cpu.c:52-56). */
constexpr unsigned D_MIN = 3;

/* SplitMix64 (G. Steele, D. Lea, C. Flood, "Fast splittable pseudorandom
 * number generators", OOPSLA 2014): the per-work-item seeds. */
uint64_t splitmix64(uint64_t *s)
{
	uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
	return z ^ (z >> 31);
}

} /* namespace */

extern "C" {

/* Work sizes the reference picks for `rows` grid rows with no work-size
 * options: gws and rows per work item. Returns -2 (PP_INVALID_ARGS) when
 * the grid has fewer than three rows, where the reference divides by
 * zero. */
int ppr_worksizes(unsigned rows, unsigned long *gws, unsigned long *rpw)
{
	const unsigned long max_gws = rows / D_MIN;
	if (max_gws == 0) return -2;
	unsigned long r = rows / max_gws;
	if ((rows % max_gws > 0) && ((max_gws - 1) * (r + 1) < rows - D_MIN)) r++;
	*gws = max_gws;
	*rpw = r;
	return 0;
}

/* A simulation of the reference's CPU algorithm: its buffers, its work
 * sizes and its model constants. */
struct ppr_sim {
	uint32_t params[13];
	uint32_t max_agents, max_iters, iter;
	unsigned long gws, rpw;
	int threads;
	void *agents, *cells, *stats;
	std::vector<uint64_t> seeds;
};

static void set_constants(const ppr_sim *s)
{
	const uint32_t *params = s->params;
	ocl::init_sheep = params[0];
	ocl::sheep_gain = params[1];
	ocl::sheep_thr = params[2];
	ocl::sheep_prob = params[3];
	ocl::init_wolves = params[4];
	ocl::wolves_gain = params[5];
	ocl::wolves_thr = params[6];
	ocl::wolves_prob = params[7];
	ocl::grass_restart = params[8];
	ocl::grid_x = params[9];
	ocl::grid_y = params[10];
	ocl::iters = s->max_iters;
	ocl::max_agents = s->max_agents;
	ocl::rows_per_workitem = (unsigned) s->rpw;
}

void ppr_destroy(ppr_sim *s)
{
	if (!s) return;
	free(s->agents);
	free(s->cells);
	free(s->stats);
	delete s;
}

/* Create a simulation and run the reference's init kernel (stats row 0).
 * params are the 13 PPParameters fields in their order
 * (pp_common.in.h:129-157); max_iters bounds the iterations that may be
 * stepped (the stats buffer holds max_iters + 1 rows, as the reference's);
 * max_agents agent slots (the reference's default 16777216 when 0, option
 * -m, pp_cpu.c:30-36); `threads` host threads (all when <= 0). *rc is 0,
 * -2 (grid below three rows), -3 (no memory) or -8 (initial agents do not
 * fit). Only one simulation may be stepped at a time per process, and not
 * from two threads at once: the model constants are process-wide, as the
 * reference's compiled-in -D values. */
ppr_sim *ppr_create(const uint32_t *params, uint64_t seed, uint32_t max_iters,
	uint32_t max_agents, int threads, int *rc)
{
	unsigned long gws = 0, rpw = 0;
	*rc = 0;
	if (ppr_worksizes(params[10], &gws, &rpw) != 0) {
		*rc = -2;
		return nullptr;
	}
	const uint32_t slots = max_agents ? max_agents : 16777216u;
	if ((uint64_t) params[0] + params[4] > slots) {
		*rc = -8;
		return nullptr;
	}
	/* the last work item of init places its agents from index (its agent
	 * count) x gid (pp_cpu.cl:361-371) */
	const uint64_t last = (uint64_t) (params[0] - params[0] / gws * (gws - 1))
		+ (params[4] - params[4] / gws * (gws - 1));
	if (last * gws > slots) {
		*rc = -8;
		return nullptr;
	}
	ppr_sim *s = new ppr_sim();
	memcpy(s->params, params, sizeof(s->params));
	s->max_agents = slots;
	s->max_iters = max_iters;
	s->iter = 0;
	s->gws = gws;
	s->rpw = rpw;
	s->threads = threads > 0 ? threads : omp_get_max_threads();
	const uint64_t cells = (uint64_t) params[9] * params[10];
	s->agents = calloc(slots, ppr_sizeof_agent());
	s->cells = calloc(cells, ppr_sizeof_cell());
	s->stats = calloc((size_t) max_iters + 1, ppr_sizeof_stats());
	if (!s->agents || !s->cells || !s->stats) {
		ppr_destroy(s);
		*rc = -3;
		return nullptr;
	}
	s->seeds.resize(gws);
	uint64_t sm = seed;
	for (unsigned long g = 0; g < gws; g++) {
		uint64_t x = splitmix64(&sm);
		s->seeds[g] = x ? x : 0x9E3779B97F4A7C15ULL;   /* xorshift needs x != 0 */
	}
	set_constants(s);
	void *sd = s->seeds.data();
	const long G = (long) gws;
#pragma omp parallel for num_threads(s->threads) schedule(static)
	for (long g = 0; g < G; g++)
		ppr_kernel_init(s->agents, s->cells, s->stats, sd, (unsigned long) g, gws);
	return s;
}

/* Stats row `iter` (seven uint32: sheep, wolves, grass, sheep_en,
 * wolves_en, grass_en, errors, the reference's PPStatisticsOcl with its
 * 32-bit sums) into out. */
void ppr_row(const ppr_sim *s, uint32_t iter, uint32_t *out)
{
	memcpy(out, (const char *) s->stats + (size_t) iter * ppr_sizeof_stats(),
		ppr_sizeof_stats());
}

/* n more iterations (ppc_simulate's loop body, pp_cpu.c:637-671); rows
 * (n x 7 uint32, may be NULL) receives their stats. Returns 0, or -2 past
 * max_iters. */
int ppr_step(ppr_sim *s, uint32_t n, uint32_t *rows)
{
	if ((uint64_t) s->iter + n > s->max_iters) return -2;
	set_constants(s);
	void *sd = s->seeds.data();
	const unsigned long gws = s->gws;
	const long G = (long) gws;
	for (uint32_t k = 0; k < n; k++) {
		const uint32_t it = ++s->iter;
		for (unsigned t = 0; t < s->rpw; t++) {
#pragma omp parallel for num_threads(s->threads) schedule(static)
			for (long g = 0; g < G; g++)
				ppr_kernel_step1(s->agents, s->cells, sd, t, (unsigned long) g, gws);
		}
		for (unsigned t = 0; t < s->rpw; t++) {
#pragma omp parallel for num_threads(s->threads) schedule(static)
			for (long g = 0; g < G; g++)
				ppr_kernel_step2(s->agents, s->cells, sd, s->stats, it, t,
					(unsigned long) g, gws);
		}
		if (rows) ppr_row(s, it, rows + 7 * (size_t) k);
	}
	return 0;
}

int ppr_threads(const ppr_sim *s) { return s->threads; }

/* The reference's agent and cell records as its kernels lay them out
 * (pp_cpu.cl:60-110): energy u16, type u8, action u8, next u32; grass u32,
 * first agent u32. */
struct ref_agent { uint16_t energy; uint8_t type, action; uint32_t next; };
struct ref_cell { uint32_t grass, first; };

/* Runs the reference's step2 kernel (actions and stats) once, for iteration
 * 1, over a grid of grid_x x 3 cells (one work item, three turns) whose
 * cells hold given agent lists. Agent i sits in cell cell_of[i] with
 * energy[i] and type[i] (0 sheep, 1 wolf), having moved (action flag set,
 * as step1 leaves it); a cell's list holds its agents in array order.
 * grass_in/grass_out are the 3 grid_x countdowns. On return, out_energy /
 * out_type hold every cell's list after the step, cell by cell in list
 * order (at most max_out entries), out_count[c] the length of cell c's list,
 * and stats7 the step's stats row (sheep, wolves, grass, sheep_en,
 * wolves_en, grass_en, errors). With the kernels compiled with shuffling
 * off (MAX_AGENT_SHUF 1) the list order is the acting order, so a test can
 * set the outcome of every draw by using reproduction probabilities of 0
 * or 100. Returns 0, -2 (params[10] is not 3 or grid_x differs), -3 (no
 * memory) or -8 (more than max_out agents after the step). */
int ppr_step2_cells(const uint32_t *params, uint32_t n, const uint32_t *cell_of,
	const uint16_t *energy, const uint8_t *type, const uint32_t *grass_in,
	uint32_t max_out, uint16_t *out_energy, uint8_t *out_type,
	uint32_t *out_count, uint32_t *grass_out, uint32_t *stats7)
{
	if (params[10] != 3 || ppr_sizeof_agent() != sizeof(ref_agent)
		|| ppr_sizeof_cell() != sizeof(ref_cell))
		return -2;
	ppr_sim s{};
	memcpy(s.params, params, sizeof(s.params));
	s.max_agents = 1u << 22;
	s.max_iters = 1;
	s.gws = 1;
	s.rpw = 3;
	const uint32_t cells = params[9] * 3;
	std::vector<ref_agent> agents(s.max_agents);
	std::vector<ref_cell> cl(cells);
	std::vector<uint32_t> stats(7 * 2, 0);
	uint64_t seed = 0x5EED;
	if (n >= s.max_agents) return -8;
	for (uint32_t c = 0; c < cells; c++) {
		cl[c].grass = grass_in[c];
		cl[c].first = 0xffffffffu;
	}
	for (uint32_t k = n; k-- > 0;) {
		ref_agent &a = agents[k];
		a.energy = energy[k];
		a.type = type[k];
		a.action = 1;
		a.next = cl[cell_of[k]].first;
		cl[cell_of[k]].first = k;
	}
	set_constants(&s);
	for (unsigned t = 0; t < 3; t++)
		ppr_kernel_step2(agents.data(), cl.data(), &seed, stats.data(), 1, t, 0, 1);
	uint32_t o = 0;
	for (uint32_t c = 0; c < cells; c++) {
		uint32_t k = 0;
		for (uint32_t a = cl[c].first; a != 0xffffffffu; a = agents[a].next, k++) {
			if (o >= max_out) return -8;
			out_energy[o] = agents[a].energy;
			out_type[o] = agents[a].type;
			o++;
		}
		out_count[c] = k;
		grass_out[c] = cl[c].grass;
	}
	memcpy(stats7, stats.data() + 7, 7 * sizeof(uint32_t));
	return 0;
}

/* A whole run: iters iterations (the parameter file's own when 0), stats
 * rows 0..iters into stats_out ((iters + 1) x 7 uint32). Returns ppr_create's
 * codes. */
int ppr_run(const uint32_t *params, uint64_t seed, uint32_t iters,
	uint32_t max_agents, int threads, uint32_t *stats_out)
{
	const uint32_t n = iters ? iters : params[12];
	int rc = 0;
	ppr_sim *s = ppr_create(params, seed, n, max_agents, threads, &rc);
	if (!s) return rc;
	ppr_row(s, 0, stats_out);
	rc = ppr_step(s, n, stats_out + 7);
	ppr_destroy(s);
	return rc;
}

}
