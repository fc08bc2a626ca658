/*
 * pp_host.c -- parameters file, validation and stats file of the drop-in
 * surface.
 *
 *   pp_load_params  follows opencl/pp/pp_common.c:39-195: whitespace-
 *                   separated `KEY = value` records read with the same
 *                   `%s = %d` scan, all 12 keys required (check mask 0xfff,
 *                   pp_common.c:169), repeated keys and unknown keys
 *                   rejected with PP_INVALID_PARAMS_FILE, a missing file
 *                   with PP_UNABLE_TO_OPEN_PARAMS_FILE.
 *   pp_stats_save   follows opencl/pp/pp_common.c:205-240: one line per
 *                   row, "%d\t%d\t%d\t%f\t%f\t%f\n", means computed as
 *                   float(sum) / float(count), 0.0 when the count is 0, and
 *                   the mean countdown as float(sum) / float(grid_xy).
 */
#include <stdio.h>
#include <string.h>
#include <stdarg.h>
#include <stdlib.h>

#include "../../include/pphpc.h"

static void set_msg(char *buf, size_t len, const char *fmt, ...)
{
	if (!buf || !len) return;
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, len, fmt, ap);
	va_end(ap);
}

static const char *const KEYS[12] = {
	"INIT_SHEEP", "SHEEP_GAIN_FROM_FOOD", "SHEEP_REPRODUCE_THRESHOLD",
	"SHEEP_REPRODUCE_PROB", "INIT_WOLVES", "WOLVES_GAIN_FROM_FOOD",
	"WOLVES_REPRODUCE_THRESHOLD", "WOLVES_REPRODUCE_PROB", "GRASS_RESTART",
	"GRID_X", "GRID_Y", "ITERS"
};

static uint32_t *field_of(PPParameters *p, int k)
{
	switch (k) {
	case 0: return &p->init_sheep;
	case 1: return &p->sheep_gain_from_food;
	case 2: return &p->sheep_reproduce_threshold;
	case 3: return &p->sheep_reproduce_prob;
	case 4: return &p->init_wolves;
	case 5: return &p->wolves_gain_from_food;
	case 6: return &p->wolves_reproduce_threshold;
	case 7: return &p->wolves_reproduce_prob;
	case 8: return &p->grass_restart;
	case 9: return &p->grid_x;
	case 10: return &p->grid_y;
	default: return &p->iters;
	}
}

int pp_load_params(PPParameters *params, const char *filename, char *errmsg,
	size_t errlen)
{
	const char *fn = filename ? filename : "config.txt";
	FILE *fp = fopen(fn, "r");
	if (!fp) {
		set_msg(errmsg, errlen, "Unable to open file \"%s\"", fn);
		return PP_UNABLE_TO_OPEN_PARAMS_FILE;
	}
	PPParameters p;
	memset(&p, 0, sizeof(p));
	char key[100];
	int value;
	unsigned check = 0;
	int rc = PP_SUCCESS;
	for (;;) {
		int got = fscanf(fp, "%99s = %d", key, &value);
		if (got == EOF) break;
		if (got != 2) {
			set_msg(errmsg, errlen, "Malformed record in parameters file");
			rc = PP_INVALID_PARAMS_FILE;
			break;
		}
		int k;
		for (k = 0; k < 12; k++)
			if (strcmp(key, KEYS[k]) == 0) break;
		if (k == 12) {
			set_msg(errmsg, errlen,
				"Invalid parameter '%s' in parameters file", key);
			rc = PP_INVALID_PARAMS_FILE;
			break;
		}
		if (check & (1u << k)) {
			set_msg(errmsg, errlen, "Repeated parameters in parameters file");
			rc = PP_INVALID_PARAMS_FILE;
			break;
		}
		*field_of(&p, k) = (uint32_t) value;
		check |= 1u << k;
	}
	fclose(fp);
	if (rc == PP_SUCCESS && check != 0x0fffu) {
		set_msg(errmsg, errlen,
			"Insufficient parameters in parameters file (check=%x)", check);
		rc = PP_INVALID_PARAMS_FILE;
	}
	if (rc == PP_SUCCESS) {
		p.grid_xy = p.grid_x * p.grid_y;
		*params = p;
	}
	return rc;
}

int pp_params_check(const PPParameters *p, char *errmsg, size_t errlen)
{
	if (!p) return PP_INVALID_ARGS;
	if (p->grid_x == 0 || p->grid_y == 0 || p->grid_x > 65535
		|| p->grid_y > 65535) {
		set_msg(errmsg, errlen, "grid sides must be in 1..65535");
		return PP_INVALID_ARGS;
	}
	uint64_t cells = (uint64_t) p->grid_x * p->grid_y;
	if (cells >= (1ull << 30)) {
		set_msg(errmsg, errlen, "grid must have fewer than 2^30 cells");
		return PP_INVALID_ARGS;
	}
	if (p->grass_restart < 1 || p->grass_restart > 32767) {
		set_msg(errmsg, errlen, "GRASS_RESTART must be in 1..32767");
		return PP_INVALID_ARGS;
	}
	if (p->sheep_reproduce_prob > 100 || p->wolves_reproduce_prob > 100) {
		set_msg(errmsg, errlen, "reproduction probabilities must be <= 100");
		return PP_INVALID_ARGS;
	}
	if (p->sheep_gain_from_food > (1u << 24)
		|| p->wolves_gain_from_food > (1u << 24)) {
		set_msg(errmsg, errlen, "gains must be <= 2^24");
		return PP_INVALID_ARGS;
	}
	if ((uint64_t) p->init_sheep + p->init_wolves >= (1ull << 31)) {
		set_msg(errmsg, errlen, "too many initial agents");
		return PP_INVALID_ARGS;
	}
	return PP_SUCCESS;
}

int pp_stats_format_row(char *buf, size_t len, const PPStatistics *s,
	const PPParameters *params)
{
	uint32_t cells = params->grid_x * params->grid_y;
	float ms = s->sheep > 0 ? (float) s->sheep_en / (float) s->sheep : 0.0f;
	float mw = s->wolves > 0 ? (float) s->wolves_en / (float) s->wolves : 0.0f;
	float mg = (float) s->grass_en / (float) cells;
	return snprintf(buf, len, "%d\t%d\t%d\t%f\t%f\t%f", (int) s->sheep,
		(int) s->wolves, (int) s->grass, ms, mw, mg);
}

int pp_stats_save(const char *filename, const PPStatistics *stats,
	uint32_t n_rows, const PPParameters *params)
{
	const char *fn = filename ? filename : "stats.txt";
	FILE *fp = fopen(fn, "w");
	if (!fp) return PP_UNABLE_SAVE_STATS;
	char line[256];
	for (uint32_t i = 0; i < n_rows; i++) {
		pp_stats_format_row(line, sizeof(line), &stats[i], params);
		if (fprintf(fp, "%s\n", line) < 0) {
			fclose(fp);
			return PP_UNABLE_SAVE_STATS;
		}
	}
	if (fclose(fp) != 0) return PP_UNABLE_SAVE_STATS;
	return PP_SUCCESS;
}

/* One iteration of the debugging dump of pp_gpu's PPG_DUMP mode
 * (opencl/pp/pp_gpu.c:415-555), appended to two text files in its line
 * formats:
 *   agents: "\nIter %d, max_agents_iter=%d, ..." then, per agent k of the
 *           canonical array, "[%4d] %016lx: (%4d, %4d) type=%d energy=%d"
 *           with the reference's 64-bit packing x << 48 | y << 32 |
 *           type << 16 | energy (16 low bits; no hash);
 *   cells:  "\nIteration %d" then, per cell, "(x, y) -> (first, last) ...
 *           [Grass: countdown]", first = last = the pool size for an empty
 *           cell, or "(x, y) -> (-, -) [Grass: countdown]" for the initial
 *           state (iteration -1).
 * dump_type 0x10 keeps only cells holding agents (and 0x01, only live
 * agents, changes nothing: the state holds live agents only). Indices are
 * positions in the state after the iteration's actions. */
int pp_sim_dump(pp_sim *sim, int dump_type, const char *agents_path,
	const char *cells_path)
{
	if (!sim || !agents_path || !cells_path) return PP_INVALID_ARGS;
	uint32_t it = 0, na = 0, cap = 0;
	int rc = pp_sim_info(sim, &it, &na, &cap);
	if (rc) return rc;
	uint32_t n = 0;
	rc = pp_sim_get_state(sim, NULL, NULL, 0, &n, NULL);
	if (rc) return rc;
	PPParameters p;
	rc = pp_sim_params(sim, &p);
	if (rc) return rc;
	const uint32_t cells = p.grid_x * p.grid_y;
	uint32_t *cell = (uint32_t *) malloc(sizeof(uint32_t) * (n ? n : 1));
	uint32_t *en = (uint32_t *) malloc(sizeof(uint32_t) * (n ? n : 1));
	uint16_t *grass = (uint16_t *) malloc(sizeof(uint16_t) * cells);
	uint32_t *first = (uint32_t *) malloc(sizeof(uint32_t) * cells);
	uint32_t *last = (uint32_t *) malloc(sizeof(uint32_t) * cells);
	FILE *fa = NULL, *fc = NULL;
	if (!cell || !en || !grass || !first || !last) {
		rc = PP_OUT_OF_RESOURCES;
		goto done;
	}
	rc = pp_sim_get_state(sim, cell, en, n, &n, grass);
	if (rc) goto done;
	fa = fopen(agents_path, "a");
	fc = fopen(cells_path, "a");
	if (!fa || !fc) {
		rc = PP_UNABLE_SAVE_STATS;
		goto done;
	}
	const int iter = it == 0 ? -1 : (int) it;
	fprintf(fa, "\nIter %d, max_agents_iter=%u, gws_reduce_agent1=%u, "
		"gws_action_ag=%u, gws_mov_ag=%u\n", iter, cap, n, n, n);
	for (uint32_t k = 0; k < n; k++) {
		const uint32_t x = cell[k] % p.grid_x, y = cell[k] / p.grid_x;
		const uint32_t type = en[k] >> 31, e = en[k] & 0x7fffffffu;
		const unsigned long long ag = ((unsigned long long) x << 48)
			| ((unsigned long long) y << 32) | ((unsigned long long) type << 16)
			| (e & 0xffffu);
		fprintf(fa, "[%4u] %016llx: (%4u, %4u) type=%u energy=%u\n",
			k, ag, x, y, type, e);
	}
	for (uint32_t c = 0; c < cells; c++) first[c] = last[c] = cap;
	for (uint32_t k = 0; k < n; k++) {
		if (first[cell[k]] == cap) first[cell[k]] = k;
		last[cell[k]] = k;
	}
	fprintf(fc, "\nIteration %d\n", iter);
	int blank_line = 0;
	for (uint32_t c = 0; c < cells; c++) {
		if (!(dump_type & 0x10) || (iter != -1 && first[c] != cap)) {
			if (blank_line) fprintf(fc, "\n");
			blank_line = 0;
			if (iter != -1)
				fprintf(fc, "(%u, %u) -> (%u, %u) %s [Grass: %u]\n",
					c % p.grid_x, c / p.grid_x, first[c], last[c],
					first[c] != last[c] ? "More than 1 agent present" : "",
					(unsigned) grass[c]);
			else
				fprintf(fc, "(%u, %u) -> (-, -) [Grass: %u]\n",
					c % p.grid_x, c / p.grid_x, (unsigned) grass[c]);
		} else {
			blank_line = 1;
		}
	}
	if (ferror(fa) || ferror(fc)) rc = PP_UNABLE_SAVE_STATS;
done:
	if (fa && fclose(fa) != 0) rc = PP_UNABLE_SAVE_STATS;
	if (fc && fclose(fc) != 0) rc = PP_UNABLE_SAVE_STATS;
	free(cell);
	free(en);
	free(grass);
	free(first);
	free(last);
	return rc;
}

const char *pp_version(void)
{
	return "pphpc_gb300 0.1 (sm_103a)";
}
