/*
 * pp_cpu_port.c -- C/OpenMP restatement of the reference's CPU simulation
 * (opencl/pp/pp_cpu.cl + opencl/pp/pp_cpu.c), used as the CPU baseline and
 * as the reference-semantics side of the statistical comparison.
 *
 * TEST AND BASELINE INFRASTRUCTURE ONLY: never linked by the product.
 *
 * The reference's CPU path cannot be built here (it needs an OpenCL CPU
 * runtime, cf4ocl2, cl_ops and GLib). This file restates its algorithm:
 *   - cells hold a grass countdown and the head of a singly linked agent
 *     list; agents hold energy, type, an "action pending" flag and the next
 *     link (pp_cpu.cl:123-168);
 *   - init: work-item g initialises its own block of cells and places its
 *     share of the sheep and wolves uniformly in that block
 *     (pp_cpu.cl:333-463);
 *   - step1, per row: grass countdown, then each agent not yet moved this
 *     iteration dies if energy <= 1, else loses 1 energy and random-walks
 *     to one of 5 cells, relinking into the destination list
 *     (pp_cpu.cl:477-580, random_walk pp_cpu.cl:268-320);
 *   - step2, per row: Fisher-Yates shuffle of each cell's list
 *     (pp_cpu.cl:236-259,636-684), then agents act in list order: sheep
 *     eat live grass; wolves eat the first sheep of the list (acted or
 *     not); every agent may reproduce into a slot found by random probing
 *     of the agent pool (alloc_ag_idx, pp_cpu.cl:182-225); newborns join
 *     the list after the cell is done (pp_cpu.cl:596-866);
 *   - rows are processed in "turns" so rows handled at the same time are
 *     at least 3 apart (PPC_D_MIN, pp_cpu.c:56; worksizes pp_cpu.c:230-334),
 *     which is what makes the parallel version race-free; work-items run
 *     as OpenMP threads.
 * The reference's RNG (cl_ops, unpinned) is not available; each work-item
 * uses its own xorshift64* generator (Vigna, "An experimental exploration
 * of Marsaglia's xorshift generators, scrambled", 2016), seeded from the
 * run seed and the work-item index by SplitMix64.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define END_OF_LIST 0xffffffffu
#define MAX_ALLOC_ATTEMPTS 500
#define MAX_SHUF 256
#define D_MIN 3

typedef struct {
	uint32_t init_sheep, sheep_gain, sheep_thr, sheep_prob;
	uint32_t init_wolves, wolves_gain, wolves_thr, wolves_prob;
	uint32_t grass_restart, grid_x, grid_y, grid_xy, iters;
} pcp_params;

typedef struct {
	uint32_t sheep, wolves, grass, errors;
	uint64_t sheep_en, wolves_en, grass_en;
} pcp_stats;

/* in: energy (16 bits, as the reference's ushort) | type << 16 |
 * action << 24; 0 means a free slot. */
typedef struct { uint32_t in; uint32_t next; } agent_t;
typedef struct { uint32_t grass; uint32_t head; } cell_t;

#define EN(a) ((a).in & 0xffffu)
#define TYPE(a) (((a).in >> 16) & 0xffu)
#define ACTION(a) ((a).in >> 24)
#define MK(en, type, act) (((uint32_t) (en) & 0xffffu) | ((uint32_t) (type) << 16) | ((uint32_t) (act) << 24))

typedef struct pcp_state {
	pcp_params p;
	uint32_t gws, rows_per_item, max_agents;
	cell_t *cells;
	agent_t *agents;
	uint64_t *rng;
	uint32_t iter;
	int threads;
} pcp_state;

static uint64_t splitmix64(uint64_t *x)
{
	uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

static inline uint32_t rnd(uint64_t *s)
{
	uint64_t x = *s;
	x ^= x >> 12;
	x ^= x << 25;
	x ^= x >> 27;
	*s = x;
	return (uint32_t) ((x * 0x2545F4914F6CDD1Dull) >> 32);
}

static inline uint32_t rnd_int(uint64_t *s, uint32_t n)
{
	return (uint32_t) (((uint64_t) rnd(s) * n) >> 32);
}

static void rem_from_cell(pcp_state *st, uint32_t cell, uint32_t ag, uint32_t prev)
{
	if (prev == END_OF_LIST) st->cells[cell].head = st->agents[ag].next;
	else st->agents[prev].next = st->agents[ag].next;
}

static void add_to_cell(pcp_state *st, uint32_t ag, uint32_t cell)
{
	st->agents[ag].next = st->cells[cell].head;
	st->cells[cell].head = ag;
}

static uint32_t random_walk(pcp_state *st, uint64_t *rng, uint32_t cell)
{
	uint32_t GX = st->p.grid_x, GY = st->p.grid_y;
	uint32_t dir = rnd_int(rng, 5);
	uint32_t x = cell % GX, y = cell / GX;
	switch (dir) {
	case 1: x = (x + 1 < GX) ? x + 1 : 0; break;
	case 2: x = (x > 0) ? x - 1 : GX - 1; break;
	case 3: y = (y + 1 < GY) ? y + 1 : 0; break;
	case 4: y = (y > 0) ? y - 1 : GY - 1; break;
	default: break;
	}
	return y * GX + x;
}

static uint32_t alloc_slot(pcp_state *st, uint64_t *rng)
{
	uint32_t s = rnd(rng);
	for (int attempt = 1; attempt < MAX_ALLOC_ATTEMPTS; attempt++) {
		uint32_t idx = s % st->max_agents;
		uint32_t expect = 0;
		if (__atomic_compare_exchange_n(&st->agents[idx].in, &expect, MK(0, 0, 1),
			0, __ATOMIC_ACQ_REL, __ATOMIC_RELAXED))
			return idx;
		s ^= s << 13;
		s ^= s >> 17;
		s ^= s << 5;
	}
	return END_OF_LIST;
}

static void row_range(const pcp_state *st, uint32_t g, uint32_t turn,
	uint32_t *lo, uint32_t *hi)
{
	uint32_t y = turn + g * st->rows_per_item;
	*lo = *hi = 0;
	if (y >= st->p.grid_y) return;
	*lo = y * st->p.grid_x;
	int last = (g == st->gws - 1) && (turn == st->rows_per_item - 1);
	*hi = last ? st->p.grid_xy : *lo + st->p.grid_x;
}

pcp_state *pcp_create(const pcp_params *pin, uint64_t seed, uint32_t max_agents,
	int threads)
{
	pcp_state *st = calloc(1, sizeof(*st));
	if (!st) return NULL;
	st->p = *pin;
	st->p.grid_xy = pin->grid_x * pin->grid_y;
	uint32_t n0 = pin->init_sheep + pin->init_wolves;
	st->max_agents = max_agents ? max_agents : (n0 * 4 > 1024 ? n0 * 4 : 1024);
	st->gws = pin->grid_y / D_MIN;
	if (st->gws == 0) st->gws = 1;
	st->rows_per_item = pin->grid_y / st->gws;
	if ((pin->grid_y % st->gws) && (st->gws - 1) * (st->rows_per_item + 1)
		< pin->grid_y - D_MIN)
		st->rows_per_item++;
	st->cells = malloc(sizeof(cell_t) * (size_t) st->p.grid_xy);
	st->agents = calloc(st->max_agents, sizeof(agent_t));
	st->rng = malloc(sizeof(uint64_t) * st->gws);
	if (!st->cells || !st->agents || !st->rng) {
		free(st->cells); free(st->agents); free(st->rng); free(st);
		return NULL;
	}
	st->threads = threads;
	uint64_t sm = seed;
	for (uint32_t g = 0; g < st->gws; g++) {
		st->rng[g] = splitmix64(&sm);
		if (!st->rng[g]) st->rng[g] = 1;
	}
	/* init (pp_cpu.cl:333-463): work-item g owns a block of cells and the
	 * agents it places; agent slots are a contiguous block per item. */
	uint32_t gws = st->gws, C = st->p.grid_xy;
	uint32_t cpw = (C + gws - 1) / gws;
	#pragma omp parallel for num_threads(threads) schedule(static)
	for (uint32_t g = 0; g < gws; g++) {
		uint64_t *rng = &st->rng[g];
		uint32_t c0 = g * cpw, c1 = (g + 1) * cpw < C ? (g + 1) * cpw : C;
		if (c0 > C) c0 = C;
		uint32_t ns = st->p.init_sheep / gws, nw = st->p.init_wolves / gws;
		if (g == gws - 1) {
			ns = st->p.init_sheep - ns * (gws - 1);
			nw = st->p.init_wolves - nw * (gws - 1);
		}
		for (uint32_t c = c0; c < c1; c++) {
			uint32_t alive = rnd_int(rng, 2);
			st->cells[c].grass = alive ? 0 : 1 + rnd_int(rng, st->p.grass_restart);
			st->cells[c].head = END_OF_LIST;
		}
		uint32_t base = (st->p.init_sheep / gws + st->p.init_wolves / gws) * g;
		for (uint32_t a = 0; a < ns + nw && c1 > c0; a++) {
			uint32_t wolf = a >= ns;
			uint32_t gain = wolf ? st->p.wolves_gain : st->p.sheep_gain;
			uint32_t e = rnd_int(rng, 2 * gain) + 1;
			uint32_t c = c0 + rnd_int(rng, c1 - c0);
			uint32_t idx = base + a;
			st->agents[idx].in = MK(e, wolf, 0);
			add_to_cell(st, idx, c);
		}
	}
	return st;
}

void pcp_destroy(pcp_state *st)
{
	if (!st) return;
	free(st->cells); free(st->agents); free(st->rng); free(st);
}

static void step1_range(pcp_state *st, uint64_t *rng, uint32_t lo, uint32_t hi)
{
	for (uint32_t c = lo; c < hi; c++) {
		if (st->cells[c].grass > 0) st->cells[c].grass--;
		uint32_t ag = st->cells[c].head, prev = END_OF_LIST;
		while (ag != END_OF_LIST) {
			uint32_t next = st->agents[ag].next;
			agent_t a = st->agents[ag];
			if (EN(a) <= 1 && !ACTION(a)) {
				st->agents[ag].in = 0;
				rem_from_cell(st, c, ag, prev);
			} else if (!ACTION(a)) {
				st->agents[ag].in = MK(EN(a) - 1, TYPE(a), 1);
				uint32_t dest = random_walk(st, rng, c);
				if (dest != c) {
					rem_from_cell(st, c, ag, prev);
					add_to_cell(st, ag, dest);
				} else {
					prev = ag;
				}
			} else {
				prev = ag;
			}
			ag = next;
		}
	}
}

static void shuffle(pcp_state *st, uint64_t *rng, const uint32_t *ptrs, uint32_t n)
{
	for (int i = (int) n - 1; i > 0; --i) {
		uint32_t j = rnd_int(rng, (uint32_t) i + 1);
		uint32_t t = st->agents[ptrs[i]].in;
		st->agents[ptrs[i]].in = st->agents[ptrs[j]].in;
		st->agents[ptrs[j]].in = t;
	}
}

static void step2_range(pcp_state *st, uint64_t *rng, uint32_t lo, uint32_t hi,
	pcp_stats *acc)
{
	uint32_t ptrs[MAX_SHUF];
	const pcp_params *p = &st->p;
	for (uint32_t c = lo; c < hi; c++) {
		/* shuffle in chunks of MAX_SHUF, as pp_cpu.cl:640-684 */
		uint32_t ag = st->cells[c].head, k = 0;
		for (;;) {
			if (ag == END_OF_LIST) { shuffle(st, rng, ptrs, k); break; }
			ptrs[k++] = ag;
			if (k >= MAX_SHUF) { shuffle(st, rng, ptrs, k); k = 0; }
			ag = st->agents[ag].next;
		}
		uint32_t nb_first = END_OF_LIST, nb_last = END_OF_LIST;
		ag = st->cells[c].head;
		while (ag != END_OF_LIST) {
			agent_t *A = &st->agents[ag];
			A->in &= 0x00ffffffu; /* action := 0 */
			uint32_t thr, prob;
			if (TYPE(*A) == 0) {
				if (st->cells[c].grass == 0) {
					st->cells[c].grass = p->grass_restart;
					A->in = MK(EN(*A) + p->sheep_gain, 0, 0);
				}
				acc->sheep++;
				acc->sheep_en += EN(*A);
				thr = p->sheep_thr; prob = p->sheep_prob;
			} else {
				uint32_t l = st->cells[c].head, lp = END_OF_LIST;
				while (l != END_OF_LIST) {
					uint32_t ln = st->agents[l].next;
					if (TYPE(st->agents[l]) == 0) {
						if (ACTION(st->agents[l]) == 0) {
							acc->sheep--;
							acc->sheep_en -= EN(st->agents[l]);
						}
						st->agents[l].in = 0;
						rem_from_cell(st, c, l, lp);
						A->in = MK(EN(*A) + p->wolves_gain, 1, 0);
						break;
					}
					lp = l;
					l = ln;
				}
				acc->wolves++;
				acc->wolves_en += EN(*A);
				thr = p->wolves_thr; prob = p->wolves_prob;
			}
			if (EN(*A) > thr && rnd_int(rng, 100) < prob) {
				uint32_t nid = alloc_slot(st, rng);
				if (nid != END_OF_LIST) {
					uint32_t ce = EN(*A) / 2;
					st->agents[nid].in = MK(ce, TYPE(*A), 0);
					st->agents[nid].next = nb_first;
					nb_first = nid;
					if (nb_last == END_OF_LIST) nb_last = nid;
					A->in = MK(EN(*A) - ce, TYPE(*A), 0);
					if (TYPE(*A) == 0) acc->sheep++; else acc->wolves++;
				} else {
					acc->errors++;
				}
			}
			ag = A->next;
		}
		if (nb_last != END_OF_LIST) {
			st->agents[nb_last].next = st->cells[c].head;
			st->cells[c].head = nb_first;
		}
		if (st->cells[c].grass == 0) acc->grass++;
		acc->grass_en += st->cells[c].grass;
	}
}

void pcp_stats_now(const pcp_state *st, pcp_stats *out)
{
	memset(out, 0, sizeof(*out));
	for (uint32_t c = 0; c < st->p.grid_xy; c++) {
		out->grass += st->cells[c].grass == 0;
		out->grass_en += st->cells[c].grass;
		for (uint32_t a = st->cells[c].head; a != END_OF_LIST; a = st->agents[a].next) {
			if (TYPE(st->agents[a])) { out->wolves++; out->wolves_en += EN(st->agents[a]); }
			else { out->sheep++; out->sheep_en += EN(st->agents[a]); }
		}
	}
}

int pcp_step(pcp_state *st, pcp_stats *out)
{
	const uint32_t R = st->rows_per_item, G = st->gws;
	for (uint32_t t = 0; t < R; t++) {
		#pragma omp parallel for num_threads(st->threads) schedule(dynamic, 8)
		for (uint32_t g = 0; g < G; g++) {
			uint32_t lo, hi;
			row_range(st, g, t, &lo, &hi);
			if (hi > lo) step1_range(st, &st->rng[g], lo, hi);
		}
	}
	pcp_stats tot;
	memset(&tot, 0, sizeof(tot));
	for (uint32_t t = 0; t < R; t++) {
		#pragma omp parallel num_threads(st->threads)
		{
			pcp_stats acc;
			memset(&acc, 0, sizeof(acc));
			#pragma omp for schedule(dynamic, 8)
			for (uint32_t g = 0; g < G; g++) {
				uint32_t lo, hi;
				row_range(st, g, t, &lo, &hi);
				if (hi > lo) step2_range(st, &st->rng[g], lo, hi, &acc);
			}
			#pragma omp critical
			{
				tot.sheep += acc.sheep; tot.wolves += acc.wolves;
				tot.grass += acc.grass; tot.errors += acc.errors;
				tot.sheep_en += acc.sheep_en; tot.wolves_en += acc.wolves_en;
				tot.grass_en += acc.grass_en;
			}
		}
	}
	st->iter++;
	if (out) *out = tot;
	return tot.errors ? -8 : 0;
}

int pcp_run(const pcp_params *p, uint64_t seed, uint32_t iters,
	uint32_t max_agents, int threads, pcp_stats *rows)
{
	pcp_state *st = pcp_create(p, seed, max_agents, threads);
	if (!st) return -3;
	pcp_stats_now(st, &rows[0]);
	int rc = 0;
	for (uint32_t t = 1; t <= iters; t++) {
		int r = pcp_step(st, &rows[t]);
		if (r && !rc) rc = r;
	}
	pcp_destroy(st);
	return rc;
}

int pcp_max_threads(void)
{
#ifdef _OPENMP
	return omp_get_max_threads();
#else
	return 1;
#endif
}
