/*
 * pp_oracle -- single-threaded CPU restatement of the PPHPC step.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it. The product (pphpc_gb300) never links or calls it.
 *
 * Parity status: the reference (nunofachada/pphpc) ships no tests, golden
 * vectors or known-answer files, and its RNG (cl_ops, unpinned) is not in
 * the reference tree, so whole runs cannot match the reference draw for
 * draw. This oracle implements the reference's model rules with
 * Philox4x32-10 draws and is pinned to the reference's own CPU kernels
 * (opencl/pp/pp_cpu.cl, compiled unmodified for the host by
 * oracle/ref/build_ref.py): its in-cell actions bit for bit wherever the
 * draws' outcomes can be fixed (tests/test_ref_act_pin.py), its whole
 * dynamics statistically (tests/test_stats_parity.py). The CUDA path is
 * checked bit for bit against this oracle.
 *
 * Rules followed (paths relative to the pphpc project root):
 *   init grass      opencl/pp/pp_gpu.cl:368-398, netlogo/pphpc.nlogo:27-35
 *   init agents     opencl/pp/pp_gpu.cl:406-439, netlogo/pphpc.nlogo:38-53
 *   move + death    opencl/pp/pp_gpu.cl:744-821, opencl/pp/pp_cpu.cl:268-320
 *   grass countdown opencl/pp/pp_gpu.cl:448-476, opencl/pp/pp_cpu.cl:504-505
 *   sort by cell    opencl/pp/pp_gpu.c:826-828 (stable, cell key only)
 *   actions         opencl/pp/pp_cpu.cl:596-866 (sequential in-cell order),
 *                   netlogo/pphpc.nlogo:79-90,133-149
 *   stats           opencl/pp/pp_cpu.cl:713-850, opencl/pp/pp_common.c:217-224
 */
#ifndef PP_ORACLE_H
#define PP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The fields of PPParameters (same order), then the width of the agents'
 * energy field: energy arithmetic is modulo 2^energy_bits, as the
 * reference's packed agents do it (pp_gpu.cl:150-316: 16 bits in its
 * 64-bit agents, 11 bits in its 32-bit ones); 0 means 30 bits. */
typedef struct ppo_params {
	uint32_t init_sheep, sheep_gain, sheep_thr, sheep_prob;
	uint32_t init_wolves, wolves_gain, wolves_thr, wolves_prob;
	uint32_t grass_restart, grid_x, grid_y, grid_xy, iters;
	uint32_t energy_bits;
} ppo_params;

/* Energy field mask of p (2^energy_bits - 1). */
uint32_t ppo_energy_mask(const ppo_params *p);

typedef struct ppo_stats {
	uint32_t sheep, wolves, grass, errors;
	uint64_t sheep_en, wolves_en, grass_en;
} ppo_stats;

/* Philox stream identifiers (third counter word). */
enum { PPO_STREAM_INIT_CELL = 0, PPO_STREAM_INIT_AGENT = 1,
	PPO_STREAM_MOVE = 2, PPO_STREAM_ACT = 3 };

#define PPO_TYPE_BIT 0x80000000u
#define PPO_ENERGY_MASK 0x7fffffffu

typedef struct ppo_state ppo_state;

/* Philox4x32-10 (Salmon et al., SC'11): out = bijection(ctr) under key. */
void ppo_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Philox at counters {c0+i, c1, c2, c3}, i < n: 4n words. */
void ppo_philox_fill(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
	uint32_t k0, uint32_t k1, uint32_t n, uint32_t *out);

/* Uniform integer in [0, n) from one 32-bit word: floor(w * n / 2^32). */
uint32_t ppo_draw(uint32_t w, uint32_t n);

/* Create and initialise (iteration 0). capacity = agent slots (0 = max(4 x
 * initial agents, 3 x cells) + 1024). Returns NULL on allocation failure. */
ppo_state *ppo_create(const ppo_params *p, uint64_t seed, uint32_t capacity);
void ppo_destroy(ppo_state *s);

/* Stats of the current state. */
void ppo_stats_now(const ppo_state *s, ppo_stats *out);

/* Advance one iteration; returns 0 or -8 on pool overflow. */
int ppo_step(ppo_state *s, ppo_stats *out);

/* Run iters iterations from a fresh state: iters+1 rows. Returns 0/-8. */
int ppo_run(const ppo_params *p, uint64_t seed, uint32_t iters,
	ppo_stats *rows);

uint32_t ppo_num_agents(const ppo_state *s);
uint32_t ppo_iter(const ppo_state *s);
void ppo_get_agents(const ppo_state *s, uint32_t *cell, uint32_t *en);
void ppo_get_grass(const ppo_state *s, uint16_t *grass);

/* Phase functions over caller arrays (for kernel-level checks). */
/* Move of iteration `iter`: dead agents get cell = grid_xy. An agent's
 * draw uses its cell and its rank among the earlier entries of that cell. */
void ppo_move(const ppo_params *p, uint64_t seed, uint32_t iter, uint32_t n,
	const uint32_t *cell_in, const uint32_t *en_in,
	uint32_t *cell_out, uint32_t *en_out);
/* Stable sort by key (keys <= max_key). */
void ppo_sort(uint32_t n, const uint32_t *k_in, const uint32_t *v_in,
	uint32_t *k_out, uint32_t *v_out, uint32_t max_key);
/* Grass countdown in place. */
void ppo_grass(uint32_t n_cells, uint16_t *grass);
/* Actions of iteration `iter` over a cell-sorted array of n live agents
 * (grass already decremented). Writes the compacted survivors+newborns
 * to cell_out/en_out (capacity cap) and returns the count, or -8 if it
 * exceeds cap. */
int64_t ppo_act(const ppo_params *p, uint64_t seed, uint32_t iter,
	uint32_t n, const uint32_t *cell, const uint32_t *en, uint16_t *grass,
	uint32_t *cell_out, uint32_t *en_out, uint32_t cap);

/* Actions of one cell's m agents, given by rank j (0..m-1): type | energy
 * en[j], priority prio[j], reproduction draw dice[j] in [0, 100); *grass is
 * the cell's countdown (updated). The agents act in increasing (priority,
 * rank) order, run as the reference's sequential scan of the cell's list.
 * Out per rank: fin (final energy), kid/haskid (newborn energy, presence),
 * eaten. */
void ppo_act_cell(const ppo_params *p, uint32_t m, const uint32_t *en,
	const uint32_t *prio, const uint32_t *dice, uint32_t *grass,
	uint32_t *fin, uint32_t *kid, uint8_t *haskid, uint8_t *eaten);

#ifdef __cplusplus
}
#endif

#endif
