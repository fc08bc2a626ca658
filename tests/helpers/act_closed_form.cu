/*
 * Host build of the CUDA path's closed-form in-cell actions (act_agent,
 * pphpc_gb300/csrc/pp_act.cuh) for tests/test_act_closed_form.py, which
 * checks it on the CPU against the oracle's literal sequential scan of the
 * reference's step2 (opencl/pp/pp_cpu.cl:690-848). Test infrastructure: the
 * same function the kernels inline, compiled for the host, nothing more.
 */
#include <cstdint>
#include <vector>

#include "pp_act.cuh"

/* Cells given by offsets off[0..ncells]: per agent i, type | energy en[i],
 * priority prio[i], reproduction draw dice[i]; per cell its countdown g0[c].
 * params: sheep gain, threshold, prob, wolves gain, threshold, prob,
 * restart, energy mask. Out per agent: val (type | final energy, or type |
 * EATEN_BIT) and kid (KID_BIT | newborn energy, or 0); per cell the number
 * of agents that ate its grass. */
extern "C" void act_cells_closed_form(const uint32_t *params, uint32_t ncells,
	const uint32_t *off, const uint32_t *en, const uint32_t *prio,
	const uint32_t *dice, const uint32_t *g0, uint32_t *val, uint32_t *kid,
	uint32_t *eaters)
{
	pp::ActParams ap;
	ap.sheep_gain = params[0]; ap.sheep_thr = params[1]; ap.sheep_prob = params[2];
	ap.wolves_gain = params[3]; ap.wolves_thr = params[4]; ap.wolves_prob = params[5];
	ap.restart = params[6]; ap.emask = params[7];
	for (uint32_t c = 0; c < ncells; c++) {
		const uint32_t p = off[c], e = off[c + 1];
		std::vector<uint32_t> LV(en + p, en + e);
		/* LV is indexed from the tile's list start; here the list is the
		 * cell alone, starting at 0 */
		uint32_t n_eat = 0;
		for (uint32_t j = 0; j < e - p; j++) {
			if (pp::act_agent(j, 0, e - p, LV.data(), prio + p, ap, g0[c],
					dice[p + j], &kid[p + j]))
				n_eat++;
		}
		for (uint32_t j = 0; j < e - p; j++) val[p + j] = LV[j];
		eaters[c] = n_eat;
	}
}
