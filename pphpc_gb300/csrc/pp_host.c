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

const char *pp_version(void)
{
	return "pphpc_gb300 0.1 (sm_103a)";
}
