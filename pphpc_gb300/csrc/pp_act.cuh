/*
 * pp_act.cuh -- device logic shared by the sort pipeline (pp_kernels.cu)
 * and the fused act+move pipeline (pp_fused.cu): the random walk and its
 * inverse, the actions of an agent in its cell, stats accumulation.
 */
#pragma once

#include "pp_kernels.cuh"
#include "pp_block.cuh"

namespace pp {

/* Run-local cell reached from run-local cell lc by direction dir of the
 * 5-way random walk (0 stay, 1 +x, 2 -x, 3 +y, 4 -y; per-row and
 * per-column wrap, pp_gpu.cl:756-819). */
__device__ __forceinline__ uint32_t move_dir(const RunDev &run, uint32_t lc,
	uint32_t dir)
{
	uint32_t y = fastdiv_div(lc, run.gxdiv);
	uint32_t x = lc - y * run.gx;
	if (dir == 1) x = (x + 1 == run.gx) ? 0 : x + 1;
	else if (dir == 2) x = (x == 0) ? run.gx - 1 : x - 1;
	else if (dir == 3) y = (y + 1 == run.gy) ? 0 : y + 1;
	else if (dir == 4) y = (y == 0) ? run.gy - 1 : y - 1;
	return y * run.gx + x;
}

/* Offset from destination cell (x, y) back to the cell an agent that moved
 * in direction dir came from (the inverse of move_dir). */
__host__ __device__ __forceinline__ int32_t src_offset(uint32_t dir,
	uint32_t x, uint32_t y, uint32_t gx, uint32_t gy)
{
	switch (dir) {
	case 1: return x == 0 ? (int32_t) (gx - 1) : -1;
	case 2: return x == gx - 1 ? -(int32_t) (gx - 1) : 1;
	case 3: return y == 0 ? (int32_t) ((gy - 1) * gx) : -(int32_t) gx;
	case 4: return y == gy - 1 ? -(int32_t) ((gy - 1) * gx) : (int32_t) gx;
	default: return 0;
	}
}

/* Energy loss (modulo the energy field), death at 0 and toroidal random
 * walk of one agent of rank k in its cell (pp_gpu.cl:756-819). */
__device__ __forceinline__ void move_one(const RunDev &run, uint32_t key,
	uint32_t val, uint32_t k, uint32_t t, uint32_t dead_key,
	uint32_t &nk, uint32_t &nv)
{
	const uint32_t e1 = ((val & ENERGY_MASK) - 1) & run.emask;
	if (e1 == 0) {
		nk = dead_key;
		nv = val & TYPE_BIT;
		return;
	}
	uint32_t lc = key - run.cbase;
	u4 r = rng(run.seed_lo, run.seed_hi, lc, t, STREAM_MOVE, k);
	nk = run.cbase + move_dir(run, lc, draw(r.x, 5));
	nv = (val & TYPE_BIT) | e1;
}

__device__ __forceinline__ bool run_live(const RunDev &run, uint32_t t)
{
	return run.active && t >= 1 && t <= run.iters;
}

/* Model parameters the actions need, held in registers. */
struct ActParams {
	uint32_t sheep_gain, sheep_thr, sheep_prob;
	uint32_t wolves_gain, wolves_thr, wolves_prob;
	uint32_t restart;
	uint32_t emask;    /* energy gains are modulo the energy field */
};

/* Actions of agent j of one cell, whose list is entries [p, e) of the
 * tile's agent list; LP[i] holds the priority of the agent of rank i - p,
 * drawn from Philox({cell, t, ACT, rank}), and dice that agent's draw of
 * U[0, 100) from the same counter. This is the sequential semantics of
 * pp_cpu.cl:640-848 (agents act in increasing (priority, rank) order;
 * wolves eat the first not-yet-eaten sheep of the cell; a sheep acts only if
 * not eaten before its turn; the first acting sheep takes live grass; every
 * acting agent may reproduce) in closed form, evaluated by the agent's own
 * thread: with sb and wb the sheep and wolves before it, the k-th wolf eats
 * the k-th sheep (a wolf gains iff wb < sheep in the cell), a sheep acts
 * iff wb <= sb and is eaten iff sb < wolves in the cell, and it takes the
 * cell's live grass (g0 == 0) iff it acts and no sheep before it acts.
 * LV[i] keeps its type bit throughout, so the agents of a cell read each
 * other's types while they write their results. On return LV[j] holds type
 * | final energy, or type | EATEN_BIT, and *kid KID_BIT | the newborn's
 * energy (which is 0 for a parent of energy 1 under a threshold of 0), or 0
 * for no newborn; the result is true iff agent j eats the grass. */
__host__ __device__ __forceinline__ bool act_agent(uint32_t j, uint32_t p, uint32_t e,
	uint32_t *LV, const uint32_t *LP, const ActParams &ap, uint32_t g0,
	uint32_t dice, uint32_t *kid)
{
	const uint32_t v = LV[j], tb = v & TYPE_BIT;
	uint32_t en = v & ENERGY_MASK;
	bool acts = true, eaten = false, grass = false;
	if (e - p == 1) {
		grass = !tb && g0 == 0;
	} else {
		const uint32_t pj = LP[j];
		uint32_t S = 0, W = 0, sb = 0, wb = 0;
		for (uint32_t i = p; i < e; i++) {
			const uint32_t pi = LP[i];
			const uint32_t before = pi < pj || (pi == pj && i < j);
			if (LV[i] & TYPE_BIT) { W++; wb += before; }
			else { S++; sb += before; }
		}
		if (tb) {
			if (wb < S) en = (en + ap.wolves_gain) & ap.emask;
		} else {
			acts = wb <= sb;
			eaten = sb < W;
			grass = acts && g0 == 0;
			/* an earlier sheep i acts iff the wolves before it are no
			 * more than the sheep before it */
			for (uint32_t i = p; i < e && grass; i++) {
				const uint32_t pi = LP[i];
				if ((LV[i] & TYPE_BIT) || !(pi < pj || (pi == pj && i < j))) continue;
				uint32_t s2 = 0, w2 = 0;
				for (uint32_t q = p; q < e; q++) {
					const uint32_t pq = LP[q];
					if (pq < pi || (pq == pi && q < i)) {
						if (LV[q] & TYPE_BIT) w2++;
						else s2++;
					}
				}
				if (w2 <= s2) grass = false;
			}
		}
	}
	if (grass) en = (en + ap.sheep_gain) & ap.emask;
	const uint32_t thr = tb ? ap.wolves_thr : ap.sheep_thr;
	const uint32_t prob = tb ? ap.wolves_prob : ap.sheep_prob;
	const bool rep = acts && en > thr && dice < prob;
	const uint32_t k = rep ? en >> 1 : 0;
	LV[j] = tb | (eaten ? EATEN_BIT : en - k);
	*kid = rep ? KID_BIT | k : 0u;
	return grass;
}

struct StatAcc {
	uint32_t sheep, wolves, galive;
	uint64_t sen, wen, gen;
	__device__ void zero() { sheep = wolves = galive = 0; sen = wen = gen = 0; }
};

/* Block-reduce the per-thread stats into out[0..5] (u64, thread f writes
 * field f). Must be called by all threads of the block. */
__device__ __forceinline__ void block_stats(const StatAcc &a, uint64_t *out)
{
	__shared__ uint64_t red[6][ACT_THREADS / 32];
	uint64_t v[6] = {a.sheep, a.wolves, a.galive, a.sen, a.wen, a.gen};
	const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
	for (int f = 0; f < 6; f++) {
		v[f] = warp_sum(v[f]);
		if (lane == 0) red[f][wid] = v[f];
	}
	__syncthreads();
	if (threadIdx.x < 6) {
		uint64_t s = 0;
		for (uint32_t q = 0; q < ACT_THREADS / 32; q++) s += red[threadIdx.x][q];
		out[threadIdx.x] = s;
	}
	__syncthreads();
}

__device__ __forceinline__ void stats_atomic_add(PPStatistics *dst,
	uint32_t f, uint64_t s)
{
	if (!s) return;
	switch (f) {
	case 0: atomicAdd(&dst->sheep, (uint32_t) s); break;
	case 1: atomicAdd(&dst->wolves, (uint32_t) s); break;
	case 2: atomicAdd(&dst->grass, (uint32_t) s); break;
	case 3: atomicAdd((unsigned long long *) &dst->sheep_en, s); break;
	case 4: atomicAdd((unsigned long long *) &dst->wolves_en, s); break;
	default: atomicAdd((unsigned long long *) &dst->grass_en, s); break;
	}
}

} /* namespace pp */
