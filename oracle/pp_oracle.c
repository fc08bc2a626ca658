/*
 * pp_oracle.c -- single-threaded CPU restatement of the PPHPC step.
 *
 * TEST INFRASTRUCTURE ONLY (the checker for the CUDA path; never linked by
 * the product). The reference has no tests or golden vectors and its cl_ops
 * RNG is not in the tree, so this file restates the model rules with
 * Philox draws; pp_oracle.h gives the reference lines each phase follows
 * and how the oracle is pinned to the reference's own CPU kernels.
 *
 * State: every cell holds an ordered list of agents; stored as an array
 * stably sorted by cell (the initial agents are listed in creation order).
 * Every draw is keyed by a cell and an agent's rank k in that cell's list,
 * never by an array position, so any storage layout that keeps the lists
 * gives the same results.
 *
 * Canonical step (iteration t = 1..iters):
 *   1. move   -- agent of rank k in cell c: energy := energy - 1 modulo
 *               2^energy_bits; 0 -> dies (pp_gpu.cl:805-810); else
 *               one of 5 directions (stay, x+1, x-1, y+1,
 *               y-1, per-row toroidal wrap as in pp_gpu.cl:771-800) drawn
 *               from Philox(ctr={c, t, MOVE, k}).w0.
 *   2. grass  -- countdown > 0 -> countdown - 1 (pp_gpu.cl:465).
 *   3. sort   -- stable sort of the survivors by cell index: a cell's new
 *               list is ordered by (source cell, rank in the source list).
 *   4. act    -- per cell c, agents in increasing (priority, k) order,
 *               priority = Philox({c, t, ACT, k}).w0 for new rank k.
 *               This is the sequential semantics of pp_cpu.cl:596-866
 *               with the shuffle replaced by the priority order, run
 *               literally as the reference's scan of the cell's list
 *               (ppo_act; the CUDA path evaluates the same rules in
 *               closed form):
 *               a wolf eats the first not-yet-eaten sheep of the cell
 *               (eaten sheep may have acted already); a sheep that is not
 *               yet eaten at its turn eats the grass if countdown == 0
 *               (countdown := restart, energy += gain; every energy
 *               gain is modulo 2^energy_bits); every agent that
 *               acts then reproduces if energy > threshold and
 *               draw(Philox({c, t, ACT, k}).w1, 100) < prob: the child
 *               gets energy/2 (0 for a parent of energy 1 under a
 *               threshold of 0: the child exists all the same) and the
 *               parent keeps the rest. Newborns
 *               neither act nor are eaten in their birth iteration.
 *               Output (the cell's next list): its agents in rank order,
 *               each surviving agent followed by its newborn (if any).
 *   5. stats  -- counts and energy sums over the output array; live grass
 *               (countdown == 0) and the countdown sum over the grid.
 */
#include "pp_oracle.h"

#include <stdlib.h>
#include <string.h>

/* Built with PPO_OMP (and -fopenmp), the loops over independent agents,
 * cells and grid entries run on threads. Every draw is keyed by cell,
 * iteration and rank, the per-cell actions touch only their cell, and the
 * sums are of integers, so the results are identical to the single-threaded
 * build; only the long full-size fixture runs use it. */
#ifdef PPO_OMP
#define PPO_FOR _Pragma("omp parallel for schedule(static)")
#define PPO_FOR_DYN _Pragma("omp parallel for schedule(dynamic, 1024)")
#else
#define PPO_FOR
#define PPO_FOR_DYN
#endif

/* Philox4x32-10, Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As
 * Easy as 1, 2, 3", SC'11: round multipliers and Weyl key increments as
 * published there. */
#define PH_M0 0xD2511F53u
#define PH_M1 0xCD9E8D57u
#define PH_W0 0x9E3779B9u
#define PH_W1 0xBB67AE85u

void ppo_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
	uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
	uint32_t k0 = key[0], k1 = key[1];
	for (int r = 0; r < 10; r++) {
		if (r > 0) {
			k0 += PH_W0;
			k1 += PH_W1;
		}
		uint64_t p0 = (uint64_t) PH_M0 * c0;
		uint64_t p1 = (uint64_t) PH_M1 * c2;
		uint32_t hi0 = (uint32_t) (p0 >> 32), lo0 = (uint32_t) p0;
		uint32_t hi1 = (uint32_t) (p1 >> 32), lo1 = (uint32_t) p1;
		c0 = hi1 ^ c1 ^ k0;
		c1 = lo1;
		c2 = hi0 ^ c3 ^ k1;
		c3 = lo0;
	}
	out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

uint32_t ppo_draw(uint32_t w, uint32_t n)
{
	return (uint32_t) (((uint64_t) w * n) >> 32);
}

static void draw4(uint64_t seed, uint32_t id, uint32_t iter, uint32_t stream,
	uint32_t k, uint32_t out[4])
{
	uint32_t ctr[4] = {id, iter, stream, k};
	uint32_t key[2] = {(uint32_t) seed, (uint32_t) (seed >> 32)};
	ppo_philox(ctr, key, out);
}

struct ppo_state {
	ppo_params p;
	uint64_t seed;
	uint32_t iter;
	uint32_t cap;
	uint32_t n;          /* live agents */
	uint32_t *cell, *en; /* agents in canonical order */
	uint32_t *cell2, *en2, *cell3, *en3;
	uint16_t *grass;
	uint32_t *count;     /* grid_xy + 2 bucket counters for the sort */
};

static uint32_t energy_of(uint32_t en) { return en & PPO_ENERGY_MASK; }

uint32_t ppo_energy_mask(const ppo_params *p)
{
	uint32_t b = p->energy_bits ? p->energy_bits : 30;
	return b >= 30 ? 0x3fffffffu : (1u << b) - 1;
}
static uint32_t type_of(uint32_t en) { return en >> 31; }

ppo_state *ppo_create(const ppo_params *p, uint64_t seed, uint32_t capacity)
{
	ppo_state *s = (ppo_state *) calloc(1, sizeof(*s));
	if (!s) return NULL;
	s->p = *p;
	s->p.grid_xy = p->grid_x * p->grid_y;
	s->seed = seed;
	uint64_t n0 = (uint64_t) p->init_sheep + p->init_wolves;
	uint64_t cells = (uint64_t) p->grid_x * p->grid_y;
	uint64_t cap = capacity ? capacity
		: (4 * n0 > 3 * cells ? 4 * n0 : 3 * cells) + 1024;
	if (cap < n0) cap = n0;
	s->cap = (uint32_t) cap;
	uint32_t C = s->p.grid_xy;
	s->cell = malloc(sizeof(uint32_t) * cap);
	s->en = malloc(sizeof(uint32_t) * cap);
	s->cell2 = malloc(sizeof(uint32_t) * cap);
	s->en2 = malloc(sizeof(uint32_t) * cap);
	s->cell3 = malloc(sizeof(uint32_t) * cap);
	s->en3 = malloc(sizeof(uint32_t) * cap);
	s->grass = malloc(sizeof(uint16_t) * (size_t) C);
	s->count = malloc(sizeof(uint32_t) * ((size_t) C + 2));
	if (!s->cell || !s->en || !s->cell2 || !s->en2 || !s->cell3 || !s->en3
		|| !s->grass || !s->count) {
		ppo_destroy(s);
		return NULL;
	}
	/* Grass: alive (0) w.p. 1/2, else 1 + U[0, restart) (pp_gpu.cl:383-393). */
	PPO_FOR
	for (uint32_t c = 0; c < C; c++) {
		uint32_t r[4];
		draw4(seed, c, 0, PPO_STREAM_INIT_CELL, 0, r);
		uint32_t alive = ppo_draw(r[0], 2);
		s->grass[c] = alive ? 0
			: (uint16_t) (1 + ppo_draw(r[1], p->grass_restart));
	}
	/* Agents: sheep first, then wolves (pp_gpu.cl:415-435); each cell's
	 * list holds its agents in this creation order, i.e. the array is
	 * stably sorted by cell. */
	PPO_FOR
	for (uint32_t a = 0; a < n0; a++) {
		uint32_t r[4];
		draw4(seed, a, 0, PPO_STREAM_INIT_AGENT, 0, r);
		uint32_t x = ppo_draw(r[0], p->grid_x);
		uint32_t y = ppo_draw(r[1], p->grid_y);
		uint32_t wolf = a >= p->init_sheep;
		uint32_t gain = wolf ? p->wolves_gain : p->sheep_gain;
		uint32_t e = (1 + ppo_draw(r[2], 2 * gain)) & ppo_energy_mask(p);
		s->cell2[a] = y * p->grid_x + x;
		s->en2[a] = (wolf ? PPO_TYPE_BIT : 0) | e;
	}
	ppo_sort((uint32_t) n0, s->cell2, s->en2, s->cell, s->en, C);
	s->n = (uint32_t) n0;
	s->iter = 0;
	return s;
}

void ppo_destroy(ppo_state *s)
{
	if (!s) return;
	free(s->cell); free(s->en); free(s->cell2); free(s->en2);
	free(s->cell3); free(s->en3); free(s->grass); free(s->count);
	free(s);
}

static void agent_stats(uint32_t n, const uint32_t *en, ppo_stats *st)
{
	uint32_t sheep = 0, wolves = 0;
	uint64_t sen = 0, wen = 0;
#ifdef PPO_OMP
	_Pragma("omp parallel for schedule(static) reduction(+:sheep, wolves, sen, wen)")
#endif
	for (uint32_t i = 0; i < n; i++) {
		uint32_t e = energy_of(en[i]);
		if (type_of(en[i])) { wolves++; wen += e; }
		else { sheep++; sen += e; }
	}
	st->sheep += sheep; st->wolves += wolves;
	st->sheep_en += sen; st->wolves_en += wen;
}

void ppo_stats_now(const ppo_state *s, ppo_stats *out)
{
	memset(out, 0, sizeof(*out));
	agent_stats(s->n, s->en, out);
	uint32_t alive = 0;
	uint64_t sum = 0;
#ifdef PPO_OMP
	_Pragma("omp parallel for schedule(static) reduction(+:alive, sum)")
#endif
	for (uint32_t c = 0; c < s->p.grid_xy; c++) {
		alive += s->grass[c] == 0;
		sum += s->grass[c];
	}
	out->grass = alive;
	out->grass_en = sum;
}

void ppo_move(const ppo_params *p, uint64_t seed, uint32_t iter, uint32_t n,
	const uint32_t *cell_in, const uint32_t *en_in,
	uint32_t *cell_out, uint32_t *en_out)
{
	uint32_t GX = p->grid_x, GY = p->grid_y, C = p->grid_x * p->grid_y;
	uint32_t emask = ppo_energy_mask(p);
	/* rank[c] = agents of cell c seen so far: an agent's rank is its
	 * position in its cell's list (earlier array entries of that cell). */
	uint32_t *ks = malloc(sizeof(uint32_t) * (n ? n : 1));
	uint32_t sorted = 1;
	for (uint32_t i = 1; i < n && sorted; i++) sorted = cell_in[i - 1] <= cell_in[i];
	if (sorted) {
		/* a cell-sorted array (the simulation's state): the rank is the
		 * distance to the cell's first entry */
		for (uint32_t i = 0; i < n; i++)
			ks[i] = (i > 0 && cell_in[i] == cell_in[i - 1]) ? ks[i - 1] + 1 : 0;
	} else {
		uint32_t *rank = calloc((size_t) C + 1, sizeof(uint32_t));
		for (uint32_t i = 0; i < n; i++)
			ks[i] = cell_in[i] < C ? rank[cell_in[i]]++ : 0;
		free(rank);
	}
	PPO_FOR
	for (uint32_t i = 0; i < n; i++) {
		uint32_t en = en_in[i];
		uint32_t e = energy_of(en);
		uint32_t k = ks[i];
		uint32_t e1 = (e - 1) & emask;
		if (e1 == 0) {
			cell_out[i] = C;           /* dead: sorts after every cell */
			en_out[i] = en & PPO_TYPE_BIT;
			continue;
		}
		uint32_t r[4];
		draw4(seed, cell_in[i], iter, PPO_STREAM_MOVE, k, r);
		uint32_t dir = ppo_draw(r[0], 5);
		uint32_t x = cell_in[i] % GX, y = cell_in[i] / GX;
		switch (dir) {
		case 1: x = (x + 1 == GX) ? 0 : x + 1; break;
		case 2: x = (x == 0) ? GX - 1 : x - 1; break;
		case 3: y = (y + 1 == GY) ? 0 : y + 1; break;
		case 4: y = (y == 0) ? GY - 1 : y - 1; break;
		default: break;
		}
		cell_out[i] = y * GX + x;
		en_out[i] = (en & PPO_TYPE_BIT) | e1;
	}
	free(ks);
}

void ppo_sort(uint32_t n, const uint32_t *k_in, const uint32_t *v_in,
	uint32_t *k_out, uint32_t *v_out, uint32_t max_key)
{
	/* stable counting sort: the moved agents are nearly in key order, so
	 * its scatter runs nearly sequentially */
	uint32_t *cnt = calloc((size_t) max_key + 2, sizeof(uint32_t));
	for (uint32_t i = 0; i < n; i++) cnt[k_in[i] + 1]++;
	for (uint32_t k = 0; k <= max_key; k++) cnt[k + 1] += cnt[k];
	for (uint32_t i = 0; i < n; i++) {
		uint32_t pos = cnt[k_in[i]]++;
		k_out[pos] = k_in[i];
		v_out[pos] = v_in[i];
	}
	free(cnt);
}

void ppo_grass(uint32_t n_cells, uint16_t *grass)
{
	PPO_FOR
	for (uint32_t c = 0; c < n_cells; c++)
		if (grass[c] > 0) grass[c]--;
}

typedef struct { uint32_t prio, slot; } ord_t;

static int ord_cmp(const void *a, const void *b)
{
	const ord_t *x = a, *y = b;
	if (x->prio != y->prio) return x->prio < y->prio ? -1 : 1;
	return x->slot < y->slot ? -1 : (x->slot > y->slot);
}

void ppo_act_cell(const ppo_params *p, uint32_t m, const uint32_t *en,
	const uint32_t *prio, const uint32_t *dice, uint32_t *grass,
	uint32_t *fin, uint32_t *kid, uint8_t *haskid, uint8_t *eaten)
{
	const uint32_t emask = ppo_energy_mask(p);
	ord_t stack_ord[64];
	ord_t *ord = m <= 64 ? stack_ord : malloc(sizeof(ord_t) * m);
	for (uint32_t j = 0; j < m; j++) {
		ord[j].prio = prio[j];
		ord[j].slot = j;
		fin[j] = energy_of(en[j]);
		kid[j] = 0;
		haskid[j] = 0;
		eaten[j] = 0;
	}
	/* the reference shuffles the list (pp_cpu.cl:641-686); here the list
	 * order is (priority, rank) */
	qsort(ord, m, sizeof(ord_t), ord_cmp);
	/* The literal sequential scan of pp_cpu.cl:690-848 over the cell's
	 * list in that order: eaten[] plays the part of the reference's removal
	 * from the list (rem_ag_from_cell), so an eaten agent is skipped at its
	 * turn and by later wolves. */
	uint32_t g = *grass;
	for (uint32_t j = 0; j < m; j++) {
		uint32_t s = ord[j].slot;
		uint32_t thr, prob;
		if (eaten[s]) continue;        /* removed before its turn */
		if (type_of(en[s])) {
			/* a wolf walks the list from its head for the first sheep
			 * still in it (acted or not), removes it and gains
			 * (pp_cpu.cl:719-768) */
			for (uint32_t q = 0; q < m; q++) {
				uint32_t s2 = ord[q].slot;
				if (eaten[s2] || type_of(en[s2])) continue;
				eaten[s2] = 1;
				fin[s] = (fin[s] + p->wolves_gain) & emask;
				break;
			}
			thr = p->wolves_thr; prob = p->wolves_prob;
		} else {
			/* a sheep eats live grass (pp_cpu.cl:700-717) */
			if (g == 0) {
				g = p->grass_restart;
				fin[s] = (fin[s] + p->sheep_gain) & emask;
			}
			thr = p->sheep_thr; prob = p->sheep_prob;
		}
		/* every acting agent may reproduce (pp_cpu.cl:771-837) */
		if (fin[s] > thr && dice[s] < prob) {
			/* the child exists even at energy 0 (a parent of energy 1
			 * under a threshold of 0), as in pp_gpu.cl:948-960 */
			kid[s] = fin[s] / 2;
			fin[s] -= kid[s];
			haskid[s] = 1;
		}
	}
	*grass = g;
	if (ord != stack_ord) free(ord);
}

int64_t ppo_act(const ppo_params *p, uint64_t seed, uint32_t iter,
	uint32_t n, const uint32_t *cell, const uint32_t *en, uint16_t *grass,
	uint32_t *cell_out, uint32_t *en_out, uint32_t cap)
{
	uint32_t *fin = malloc(sizeof(uint32_t) * (n ? n : 1));   /* final energy */
	uint32_t *kid = malloc(sizeof(uint32_t) * (n ? n : 1));   /* child energy */
	uint8_t *haskid = malloc(n ? n : 1);   /* a child (its energy may be 0) */
	uint8_t *eaten = malloc(n ? n : 1);
	uint32_t *prio = malloc(sizeof(uint32_t) * (n ? n : 1));
	uint32_t *dice = malloc(sizeof(uint32_t) * (n ? n : 1));
	uint64_t out = 0;
	int64_t ret;

	/* the cells' segments of the cell-sorted array */
	uint32_t nseg = 0;
	for (uint32_t i = 0; i < n; i++) nseg += i == 0 || cell[i] != cell[i - 1];
	uint32_t *seg = malloc(sizeof(uint32_t) * ((size_t) nseg + 1));
	nseg = 0;
	for (uint32_t i = 0; i < n; i++)
		if (i == 0 || cell[i] != cell[i - 1]) seg[nseg++] = i;
	seg[nseg] = n;
	PPO_FOR_DYN
	for (uint32_t q = 0; q < nseg; q++) {
		uint32_t lo = seg[q], hi = seg[q + 1], c = cell[lo];
		uint32_t m = hi - lo;
		for (uint32_t j = 0; j < m; j++) {
			uint32_t r[4];
			draw4(seed, c, iter, PPO_STREAM_ACT, j, r);
			prio[lo + j] = r[0];
			dice[lo + j] = ppo_draw(r[1], 100);
		}
		uint32_t g = grass[c];
		ppo_act_cell(p, m, en + lo, prio + lo, dice + lo, &g, fin + lo,
			kid + lo, haskid + lo, eaten + lo);
		grass[c] = (uint16_t) g;
	}
	free(seg);
	for (uint32_t s = 0; s < n; s++) {
		uint32_t tb = en[s] & PPO_TYPE_BIT;
		if (!eaten[s]) {
			if (out < cap) { cell_out[out] = cell[s]; en_out[out] = tb | fin[s]; }
			out++;
		}
		if (haskid[s]) {
			if (out < cap) { cell_out[out] = cell[s]; en_out[out] = tb | kid[s]; }
			out++;
		}
	}
	ret = out > cap ? -8 : (int64_t) out;
	free(fin); free(kid); free(haskid); free(eaten); free(prio); free(dice);
	return ret;
}

int ppo_step(ppo_state *s, ppo_stats *out)
{
	uint32_t t = s->iter + 1, C = s->p.grid_xy;
	ppo_move(&s->p, s->seed, t, s->n, s->cell, s->en, s->cell2, s->en2);
	ppo_grass(C, s->grass);
	ppo_sort(s->n, s->cell2, s->en2, s->cell3, s->en3, C);
	uint32_t live = 0;
	while (live < s->n && s->cell3[live] < C) live++;
	int64_t m = ppo_act(&s->p, s->seed, t, live, s->cell3, s->en3, s->grass,
		s->cell, s->en, s->cap);
	s->iter = t;
	if (m < 0) {
		s->n = 0;
		if (out) { memset(out, 0, sizeof(*out)); out->errors = 1; }
		return -8;
	}
	s->n = (uint32_t) m;
	if (out) ppo_stats_now(s, out);
	return 0;
}

int ppo_run(const ppo_params *p, uint64_t seed, uint32_t iters,
	ppo_stats *rows)
{
	ppo_state *s = ppo_create(p, seed, 0);
	if (!s) return -3;
	ppo_stats_now(s, &rows[0]);
	int rc = 0;
	for (uint32_t t = 1; t <= iters && rc == 0; t++)
		rc = ppo_step(s, &rows[t]);
	ppo_destroy(s);
	return rc;
}

uint32_t ppo_num_agents(const ppo_state *s) { return s->n; }
uint32_t ppo_iter(const ppo_state *s) { return s->iter; }

void ppo_get_agents(const ppo_state *s, uint32_t *cell, uint32_t *en)
{
	memcpy(cell, s->cell, sizeof(uint32_t) * s->n);
	memcpy(en, s->en, sizeof(uint32_t) * s->n);
}

void ppo_get_grass(const ppo_state *s, uint16_t *grass)
{
	memcpy(grass, s->grass, sizeof(uint16_t) * s->p.grid_xy);
}

void ppo_philox_fill(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
	uint32_t k0, uint32_t k1, uint32_t n, uint32_t *out)
{
	uint32_t key[2] = {k0, k1};
	for (uint32_t i = 0; i < n; i++) {
		uint32_t ctr[4] = {c0 + i, c1, c2, c3};
		ppo_philox(ctr, key, out + 4 * (size_t) i);
	}
}
