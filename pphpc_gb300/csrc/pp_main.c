/*
 * pp_main.c -- command-line drop-in for the reference's pp_gpu executable
 * (opencl/pp/pp_gpu.c:1700-1946, options pp_gpu.c:310-410).
 *
 *   pp_gb300 [-p PARAMS] [-s STATS] [-r SEED] [-d DEVICE] [-m MAX_AGENTS]
 *            [-a AGENT_SIZE] [--iters N] [-i PROF_FILE] [-t TILE]
 *            [--digit-bits B] [--no-graph] [--dump TYPE]
 *
 * The reference's OpenCL tuning options (-c/--compiler, --a-rng, --a-sort,
 * --a-sort-opts, --l-*, --vw-*) are accepted with their argument and have
 * no effect here (a note goes to stderr), so existing command lines run
 * unchanged.
 *
 * -p/-s/-r/-d/-m/-a keep the reference's meaning and defaults (config.txt,
 * stats.txt, seed 0, device 0, agent pool, 64-bit agents: -a sets the
 * width of the energy field, 16 bits for 64 and 11 bits for 32, with the
 * reference's modular energy arithmetic); --iters overrides ITERS from
 * the parameters file (the reference has no such knob: -i there is the
 * profiling export, kept here as a two-column kernel-time file). --dump
 * writes dump_agents.txt and dump_cells.txt after every iteration in the
 * formats of the reference's compile-time PPG_DUMP mode (pp_gpu.c:28-47,
 * 415-555), TYPE as there (0x00, 0x01, 0x10, 0x11). The exit status is a
 * pp_error_codes value, as in the reference.
 */
#include <getopt.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../../include/pphpc.h"

static double now_s(void)
{
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return ts.tv_sec + ts.tv_nsec * 1e-9;
}

static void usage(const char *argv0)
{
	fprintf(stderr,
		"Usage: %s [-p FILE] [-s FILE] [-r SEED] [-d INDEX] [-m MAX]\n"
		"          [-a 32|64] [--iters N] [-i FILE] [-t TILE] [--digit-bits B]\n"
		"          [--no-graph] [--dump TYPE]\n",
		argv0);
}

int main(int argc, char **argv)
{
	const char *params_file = NULL, *stats_file = NULL, *prof_file = NULL;
	long long seed = 0;
	long long iters_override = -1;
	int dump_type = -1;
	pp_opts opts;
	pp_opts_default(&opts);
	long agent_size = 64;
	static struct option longopts[] = {
		{"params", required_argument, 0, 'p'},
		{"stats", required_argument, 0, 's'},
		{"rng-seed", required_argument, 0, 'r'},
		{"device", required_argument, 0, 'd'},
		{"max-agents", required_argument, 0, 'm'},
		{"agent-size", required_argument, 0, 'a'},
		{"prof-agg", required_argument, 0, 'i'},
		{"iters", required_argument, 0, 'I'},
		{"tile", required_argument, 0, 't'},
		{"digit-bits", required_argument, 0, 'D'},
		{"no-graph", no_argument, 0, 'G'},
		{"dump", required_argument, 0, 'U'},
		{"help", no_argument, 0, 'h'},
		/* the reference's OpenCL options (pp_gpu.c:310-410), without effect */
		{"compiler", required_argument, 0, 'c'},
		{"a-rng", required_argument, 0, 'X'},
		{"a-sort", required_argument, 0, 'X'},
		{"a-sort-opts", required_argument, 0, 'X'},
		{"l-def", required_argument, 0, 'X'},
		{"l-init-cell", required_argument, 0, 'X'},
		{"l-init-agent", required_argument, 0, 'X'},
		{"l-grass", required_argument, 0, 'X'},
		{"l-reduce-grass", required_argument, 0, 'X'},
		{"l-reduce-agent", required_argument, 0, 'X'},
		{"l-move-agent", required_argument, 0, 'X'},
		{"l-sort-agent", required_argument, 0, 'X'},
		{"l-find-index", required_argument, 0, 'X'},
		{"l-action-agent", required_argument, 0, 'X'},
		{"vw-grass", required_argument, 0, 'X'},
		{"vw-reduce-grass", required_argument, 0, 'X'},
		{"vw-reduce-agent", required_argument, 0, 'X'},
		{0, 0, 0, 0}
	};
	int c, li = 0;
	while ((c = getopt_long(argc, argv, "p:s:r:d:m:a:i:t:c:h", longopts, &li)) != -1) {
		switch (c) {
		case 'c':
			fprintf(stderr, "Note: -c/--compiler has no effect here (OpenCL option)\n");
			break;
		case 'X':
			fprintf(stderr, "Note: --%s has no effect here (OpenCL option)\n",
				longopts[li].name);
			break;
		case 'p': params_file = optarg; break;
		case 's': stats_file = optarg; break;
		case 'r': seed = strtoll(optarg, NULL, 0); break;
		case 'd': opts.device = atoi(optarg); break;
		case 'm': opts.max_agents = (uint32_t) strtoul(optarg, NULL, 0); break;
		case 'a': agent_size = strtol(optarg, NULL, 0); break;
		case 'i': prof_file = optarg; break;
		case 'I': iters_override = strtoll(optarg, NULL, 0); break;
		case 't': opts.tile_cells = (uint32_t) strtoul(optarg, NULL, 0); break;
		case 'D': opts.sort_digit_bits = (uint32_t) strtoul(optarg, NULL, 0); break;
		case 'G': opts.use_graph = 0; break;
		case 'U': dump_type = (int) strtol(optarg, NULL, 0); break;
		case 'h': usage(argv[0]); return PP_SUCCESS;
		default: usage(argv[0]); return PP_UNKNOWN_ARGS;
		}
	}
	if (optind < argc) {
		fprintf(stderr, "Error: This program does not accept non-option arguments.\n");
		return PP_UNKNOWN_ARGS;
	}
	if (agent_size != 32 && agent_size != 64) {
		fprintf(stderr, "Error: The -a (--agent-size) parameter must be "
			"either 32 or 64.\n");
		return PP_INVALID_ARGS;
	}
	opts.agent_size = (uint32_t) agent_size;
	char msg[256] = "";
	PPParameters params;
	int rc = pp_load_params(&params, params_file, msg, sizeof(msg));
	if (rc) {
		fprintf(stderr, "Error: %s\n", msg);
		return rc;
	}
	if (iters_override >= 0) params.iters = (uint32_t) iters_override;
	rc = pp_params_check(&params, msg, sizeof(msg));
	if (rc) {
		fprintf(stderr, "Error: %s\n", msg);
		return rc;
	}
	PPStatistics *rows = (PPStatistics *) calloc((size_t) params.iters + 1,
		sizeof(PPStatistics));
	if (!rows) return PP_OUT_OF_RESOURCES;
	double t0 = now_s();
	pp_sim *sim = NULL;
	if (agent_size == 32 && (params.grid_x > 1024 || params.grid_y > 1024)) {
		fprintf(stderr, "Error: 32-bit agents hold grid coordinates up to "
			"1023; use -a 64 for this grid.\n");
		free(rows);
		return PP_INVALID_ARGS;
	}
	rc = pp_sim_create(&params, (uint64_t) seed, &opts, &sim);
	if (rc) {
		fprintf(stderr, "Error: unable to create simulation (%d)\n", rc);
		free(rows);
		return rc;
	}
	pp_sim_stats0(sim, &rows[0]);
	double t1 = now_s();
	if (dump_type >= 0) {
		/* debugging mode: one iteration at a time, dumped after each */
		const char *fa = "dump_agents.txt", *fc = "dump_cells.txt";
		FILE *f1 = fopen(fa, "w"), *f2 = fopen(fc, "w");
		if (f1) fclose(f1);
		if (f2) fclose(f2);
		rc = (f1 && f2) ? pp_sim_dump(sim, dump_type, fa, fc) : PP_UNABLE_SAVE_STATS;
		for (uint32_t i = 0; i < params.iters && rc == PP_SUCCESS; i++) {
			rc = pp_sim_step(sim, 1, rows + 1 + i);
			if (rc == PP_SUCCESS) rc = pp_sim_dump(sim, dump_type, fa, fc);
		}
	} else {
		rc = pp_sim_step(sim, params.iters, rows + 1);
	}
	double t2 = now_s();
	if (rc == PP_OUT_OF_RESOURCES)
		fprintf(stderr, "Error: agents required above the pool limit "
			"(-m); raise it\n");
	else if (rc)
		fprintf(stderr, "Error: simulation failed (%d)\n", rc);
	pp_sim_destroy(sim);
	if (rc == PP_SUCCESS) {
		rc = pp_stats_save(stats_file, rows, params.iters + 1, &params);
		if (rc) fprintf(stderr, "Error: unable to save stats\n");
	}
	if (rc == PP_SUCCESS && prof_file) {
		FILE *fp = fopen(prof_file, "w");
		if (fp) {
			fprintf(fp, "\"init\"\t%.0f\n\"simulate\"\t%.0f\n",
				(t1 - t0) * 1e9, (t2 - t1) * 1e9);
			fclose(fp);
		}
	}
	if (rc == PP_SUCCESS)
		printf("Ellapsed time: %.4es\n", t2 - t0);
	free(rows);
	return rc;
}
