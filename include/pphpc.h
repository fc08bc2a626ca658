/*
 * pphpc_gb300 -- C ABI of the GB300-native PPHPC simulation step.
 *
 * Every entry point takes plain C types and pointers; no CUDA or framework
 * type crosses this boundary except where a function name says "dev" (a raw
 * device address as `void*`) or "stream" (a `cudaStream_t` passed as `void*`).
 * All functions return 0 (PP_SUCCESS) or a negative `pp_error_codes` value;
 * the library never calls exit().
 *
 * Reference interfaces replaced (paths relative to the pphpc project root):
 *   PPParameters       opencl/pp/pp_common.in.h:129-157
 *   PPStatistics       opencl/pp/pp_common.in.h:109-124 (sums widened to 64 bit)
 *   pp_error_codes     opencl/pp/pp_common.in.h:87-104
 *   pp_load_params     opencl/pp/pp_common.c:39-195
 *   pp_stats_save      opencl/pp/pp_common.c:205-240
 *   ppg_simulate       opencl/pp/pp_gpu.c:573-987 (split into create/step/destroy)
 *   main (pp_gpu)      opencl/pp/pp_gpu.c:1700-1946 (see pp_main.c)
 */
#ifndef PPHPC_GB300_H
#define PPHPC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Error codes: opencl/pp/pp_common.in.h:87-104, extended.             */
/* ------------------------------------------------------------------ */
enum pp_error_codes {
	PP_SUCCESS = 0,
	PP_UNKNOWN_ARGS = -1,
	PP_INVALID_ARGS = -2,
	PP_LIBRARY_ERROR = -3,
	PP_UNABLE_TO_OPEN_PARAMS_FILE = -4,
	PP_INVALID_PARAMS_FILE = -5,
	PP_UNABLE_SAVE_STATS = -6,
	PP_OUT_OF_RESOURCES = -8,
	/* Extensions of this library. */
	PP_ERR_CUDA = -9,     /* a CUDA runtime call failed                    */
	PP_ERR_TIMEOUT = -10, /* a bounded device-side wait gave up           */
	PP_ERR_CANCELLED = -11/* a served request was cancelled              */
};

#define PP_SHEEP_ID 0
#define PP_WOLF_ID 1

/* Simulation parameters: same fields and order as the reference struct
 * (opencl/pp/pp_common.in.h:129-157). `grid_xy` is derived. */
typedef struct pp_parameters {
	uint32_t init_sheep;
	uint32_t sheep_gain_from_food;
	uint32_t sheep_reproduce_threshold;
	uint32_t sheep_reproduce_prob;
	uint32_t init_wolves;
	uint32_t wolves_gain_from_food;
	uint32_t wolves_reproduce_threshold;
	uint32_t wolves_reproduce_prob;
	uint32_t grass_restart;
	uint32_t grid_x;
	uint32_t grid_y;
	uint32_t grid_xy;
	uint32_t iters;
} PPParameters;

/* Per-iteration statistics (opencl/pp/pp_common.in.h:109-124). Row k is the
 * state after k iterations. The fields are the reference's, in the
 * reference's order (errors last); the energy and countdown sums are 64-bit
 * here because the reference's 32-bit sums overflow on a 12800x12800 grid.
 * Layout (48 bytes, natural alignment): sheep 0, wolves 4, grass 8, 4 bytes
 * of padding, sheep_en 16, wolves_en 24, grass_en 32, errors 40, 4 bytes of
 * padding. */
typedef struct pp_statistics {
	uint32_t sheep;
	uint32_t wolves;
	uint32_t grass;    /* cells with countdown == 0                    */
	uint64_t sheep_en;
	uint64_t wolves_en;
	uint64_t grass_en; /* sum of grass countdowns                      */
	uint32_t errors;   /* pool-overflow events (0 in a successful run) */
} PPStatistics;

/* ------------------------------------------------------------------ */
/* Parameter file and stats file (drop-in formats).                    */
/* ------------------------------------------------------------------ */

/* Parse a `KEY = int` parameters file; all 12 keys required, repeats and
 * unknown keys rejected. Replaces pp_load_params (pp_common.c:39-195).
 * Returns PP_UNABLE_TO_OPEN_PARAMS_FILE or PP_INVALID_PARAMS_FILE on error;
 * a message is written to `errmsg` (may be NULL) of size `errlen`. */
int pp_load_params(PPParameters *params, const char *filename,
	char *errmsg, size_t errlen);

/* Validate parameters against this implementation's limits (grid sides
 * 1..65535, grid_xy < 2^30, 1 <= grass_restart <= 32767, probabilities
 * <= 100). Returns PP_SUCCESS or PP_INVALID_ARGS. */
int pp_params_check(const PPParameters *params, char *errmsg, size_t errlen);

/* Write `n_rows` stats rows as `%d\t%d\t%d\t%f\t%f\t%f\n` (sheep, wolves,
 * grass, mean sheep energy, mean wolf energy, mean countdown), the format
 * of pp_stats_save (pp_common.c:205-240). Means are computed in float as
 * the reference does. Returns PP_UNABLE_SAVE_STATS on I/O failure. */
int pp_stats_save(const char *filename, const PPStatistics *stats,
	uint32_t n_rows, const PPParameters *params);

/* Format one stats row exactly as pp_stats_save does (no newline);
 * returns the number of characters written (snprintf semantics). */
int pp_stats_format_row(char *buf, size_t len, const PPStatistics *row,
	const PPParameters *params);

/* ------------------------------------------------------------------ */
/* Single simulation (one run per launch sequence).                    */
/* ------------------------------------------------------------------ */

typedef struct pp_sim pp_sim;

typedef struct pp_opts {
	int device;             /* CUDA device ordinal (default 0)                */
	uint32_t max_agents;    /* agent pool slots; 0 = 4 x initial agents, >= 1024 */
	uint32_t tile_cells;    /* cells per act tile: 1024..8192, or 512 for the
	                           fused pipeline; 0 = choose (or autotune)    */
	uint32_t sort_digit_bits; /* radix digit width 4..8; 0 = autotune         */
	uint32_t use_graph;     /* 1: run iterations as CUDA graphs of 32, captured
	                           by the first call that runs 32 in a row (a
	                           simulation created inside a stream capture
	                           should make that call outside it); 0: launch
	                           by launch */
	uint32_t sort_pipeline; /* 1 = per-iteration sort pipeline (move, LSD radix
	                           passes over the tile bits, tile offsets, act);
	                           0 = fused act+move with a gather by destination
	                           tile (default) */
	uint32_t autotune;      /* 1 = when tile_cells is 0, measure the candidate
	                           geometries (pp_autotune) and use the fastest;
	                           0 = built-in choice */
	uint32_t ss_from;       /* focal measures: the steady state is the
	                           iterations after ss_from (default 1000) */
	uint32_t agent_size;    /* the reference's -a/--agent-size (pp_gpu.c:334,
	                           1632-1634): 64 = energy modulo 2^16 as in its
	                           64-bit agents, 32 = modulo 2^11 as in its
	                           32-bit agents (grids up to 1024 x 1024);
	                           0 = modulo 2^30 (default); else PP_INVALID_ARGS */
} pp_opts;

/* PPHPC focal measures of a run's six outputs, in the order sheep, wolves,
 * live grass, mean sheep energy, mean wolf energy, mean grass countdown
 * (the columns of the stats file): the maximum and minimum over iterations
 * 0..t with the first iteration reaching each, and the mean and sample
 * standard deviation over the steady state (iterations after ss_from).
 * Computed on the GPU as the iterations run, so a caller needs no stats
 * rows to get them. No counterpart in the reference (the measures are
 * those of Fachada et al., "Towards a standard model for research in
 * agent-based modeling and simulation", PeerJ CS 2015). */
typedef struct pp_focal {
	double max[6], min[6], ss_mean[6], ss_std[6];
	uint32_t argmax[6], argmin[6];
	uint32_t ss_n;          /* steady-state iterations counted */
	uint32_t pad;
} pp_focal;

/* Fill `opts` with defaults. */
void pp_opts_default(pp_opts *opts);

/* Allocate device state and initialise grid and agents (iteration 0) on
 * the GPU. The stats of iteration 0 are available via pp_sim_stats0.
 * Replaces the set-up half of ppg_simulate (pp_gpu.c:573-660). */
int pp_sim_create(const PPParameters *params, uint64_t seed,
	const pp_opts *opts, pp_sim **out);

/* Statistics of the initial state (row 0 of the stats file). */
int pp_sim_stats0(pp_sim *sim, PPStatistics *out);

/* Run `n_iters` iterations; row i of `out` receives the stats after
 * iteration (current + i + 1). Blocks until done. Replaces the loop of
 * ppg_simulate (pp_gpu.c:671-935). Returns PP_OUT_OF_RESOURCES if the agent
 * pool overflowed (state is then undefined). */
int pp_sim_step(pp_sim *sim, uint32_t n_iters, PPStatistics *out);

/* Same as pp_sim_step but leaves the stats in device memory: `dev_stats`
 * is a device pointer to `n_iters` PPStatistics rows; asynchronous on the
 * simulation's stream (pp_sim_stream). Overflow is reported by the next
 * pp_sim_sync. */
int pp_sim_step_async(pp_sim *sim, uint32_t n_iters, void *dev_stats);

/* Wait for the simulation's stream; returns PP_OUT_OF_RESOURCES if any
 * earlier asynchronous step overflowed the pool. */
int pp_sim_sync(pp_sim *sim);

/* Current iteration number and live agent count. */
int pp_sim_info(pp_sim *sim, uint32_t *iter, uint32_t *n_agents,
	uint32_t *capacity);

/* Copy the state out: agents in array order (`cell`, `en` = type<<31 |
 * energy; `n_max` slots), grass countdowns (grid_xy values; may be NULL). */
int pp_sim_get_state(pp_sim *sim, uint32_t *cell, uint32_t *en,
	uint32_t n_max, uint32_t *n_agents, uint16_t *grass);

/* Per-kernel timing (replaces the reference's cf4ocl event profiler,
 * pp_gpu.c:1868-1881 and --prof-agg, pp_common.c:248-260): runs n_iters
 * iterations without graph replay, with CUDA events on the simulation's
 * stream around every kernel. prof[0..4] = move, radix_pass, offsets, act,
 * finish: launches, total milliseconds and algorithmic bytes moved (minimum
 * reads plus writes of each kernel). `agent_steps` = sum of live agents at
 * the start of each iteration. n_prof must be >= 5. */
typedef struct pp_kernel_prof {
	char name[32];
	uint32_t launches;
	double total_ms;
	double bytes;
} pp_kernel_prof;

int pp_sim_profile(pp_sim *sim, uint32_t n_iters, pp_kernel_prof *prof,
	uint32_t n_prof, double *agent_steps);

/* Run n_iters iterations (graph replay) between two CUDA events on the
 * simulation's stream; *ms = elapsed device time. */
int pp_sim_time(pp_sim *sim, uint32_t n_iters, float *ms);

/* Stats rows of iterations [first_iter, first_iter + n) still held in the
 * device ring (the last ring_rows - 1 iterations). */
int pp_sim_stats_range(pp_sim *sim, uint32_t first_iter, uint32_t n,
	PPStatistics *out);

/* Bytes the simulation has copied host->device and device->host so far
 * (parameters, run tables, stats rows, status words). */
int pp_sim_io_bytes(pp_sim *sim, uint64_t *h2d, uint64_t *d2h);

/* The cudaStream_t the simulation runs on (as void*). */
void *pp_sim_stream(pp_sim *sim);

/* Write the simulation's state after its last iteration -- agents in
 * canonical order (run-local cell, type << 31 | energy), grass countdowns,
 * the iteration number, parameters and seed -- to the file `path`. A
 * simulation restored from it continues with exactly the stats and state
 * of the uninterrupted one (every draw is keyed by cell, iteration and
 * rank, none by memory layout). No counterpart in the reference (state
 * snapshot / resume is new here). */
int pp_sim_snapshot_save(pp_sim *sim, const char *path);

/* Create a simulation from a snapshot file written by pp_sim_snapshot_save.
 * pp_sim_stats0 returns the stats of the saved state and pp_sim_info the
 * saved iteration plus the iterations run since. PP_INVALID_PARAMS_FILE if
 * the file is not a snapshot. */
int pp_sim_restore(const char *path, const pp_opts *opts, pp_sim **out);

/* The simulation's parameters (as checked at creation or restore). */
int pp_sim_params(pp_sim *sim, PPParameters *out);

/* The focal measures of the iterations run so far (from iteration 0, or
 * the restored iteration). */
int pp_sim_focal(pp_sim *sim, pp_focal *out);

/* Append the state after the last iteration to two text files in the line
 * formats of pp_gpu's PPG_DUMP debugging mode (pp_gpu.c:415-555): agents
 * (index, packed agent, position, type, energy) and cells (position, first
 * and last agent index, grass countdown). dump_type as PPG_DUMP: 0x10
 * keeps only cells holding agents. The initial state (iteration 0) is
 * labelled -1, as the reference labels its dump before the first
 * iteration. */
int pp_sim_dump(pp_sim *sim, int dump_type, const char *agents_path,
	const char *cells_path);

int pp_sim_destroy(pp_sim *sim);

/* Device buffers of destroyed simulations, batches and servers stay cached
 * in the process (at most a quarter of a device's memory; environment
 * variable PP_CACHE_BYTES sets the limit, 0 disables the cache) and serve
 * the next creation on that device without driver allocations. This frees
 * the cached buffers of `device` (-1: every device); *released = bytes. */
int pp_release_cached_memory(int device, uint64_t *released);

/* ------------------------------------------------------------------ */
/* Kernel-level entry points (host buffers in and out, synchronous).   */
/* Used to check each kernel alone against the oracle.                 */
/* ------------------------------------------------------------------ */

/* Philox4x32-10 at counters {ctr0 + i, ctr1, ctr2, ctr3}, key {k0, k1}:
 * 4*n words out (i = 0..n-1). */
int pp_philox_fill(uint32_t ctr0, uint32_t ctr1, uint32_t ctr2, uint32_t ctr3,
	uint32_t k0, uint32_t k1, uint32_t n, uint32_t *out);

/* Move phase of iteration `iter` (move_agent, pp_gpu.cl:744-821): agents
 * in slot order in, moved agents out (dead ones get cell = grid_xy). */
int pp_move_host(const PPParameters *params, uint64_t seed, uint32_t iter,
	uint32_t n, const uint32_t *cell_in, const uint32_t *en_in,
	uint32_t *cell_out, uint32_t *en_out);

/* Stable LSD radix sort of (key, value) pairs whose keys are below
 * 2^key_bits (replaces the cl_ops sort call, pp_gpu.c:826-828); key_bits
 * 1..32, digit_bits 5..8 or 0 = auto. */
int pp_radix_sort_host(uint32_t n, const uint32_t *keys_in,
	const uint32_t *vals_in, uint32_t *keys_out, uint32_t *vals_out,
	uint32_t key_bits, uint32_t digit_bits);

/* Failure-detection self-test of the bounded device-side waits: n_chunks
 * (<= 4096) chunks of one launch run the finish kernel's decoupled
 * look-back, each publishing chunk + 1; prefix_out (n_chunks words, may be
 * NULL) receives each chunk's exclusive prefix. With stall_chunk >= 0 that
 * chunk never publishes: the wait behind it gives up after a bounded number
 * of polls and the call returns PP_ERR_TIMEOUT, the device staying usable;
 * with -1 it returns PP_SUCCESS and prefix_out[k] = k (k + 1) / 2. */
int pp_lookback_selftest(uint32_t n_chunks, int32_t stall_chunk,
	uint32_t *prefix_out);

/* Largest n accepted by pp_radix_sort_noalloc. */
#define PP_NOALLOC_SORT_MAX_N (1u << 22)

/* No counterpart in the reference: it exists for callers that must not
 * allocate device memory, such as an application whose device memory is
 * owned by its own pooling allocator, or a loop with a latency budget in
 * which cudaMalloc/cudaFree could synchronise the device. Same stable LSD
 * radix sort as pp_radix_sort_host (keys below 2^key_bits), but on
 * caller-owned device buffers
 * (`keys`, `vals` in; `keys_out`, `vals_out` out; the input buffers are
 * overwritten as ping-pong space) and with its scratch in a fixed array
 * inside the library (about 2 MB per GPU, held until the process exits).
 * It calls no cudaMalloc/cudaFree. Limit: n <= PP_NOALLOC_SORT_MAX_N, else
 * PP_INVALID_ARGS. The first call on a device looks up the array's device
 * address; make that first call before any stream capture. All calls share
 * the array: calls that overlap on the GPU (other streams, other threads)
 * race and must be serialised by the caller. Runs on `stream` (a
 * cudaStream_t, NULL = legacy stream) and returns after it completes. */
int pp_radix_sort_noalloc(uint32_t n, uint32_t *keys, uint32_t *vals,
	uint32_t *keys_out, uint32_t *vals_out, uint32_t key_bits,
	uint32_t digit_bits, void *stream);

/* Dense per-cell start offsets of a cell-sorted key array: off[c] = first
 * index with key >= c, for c = 0..n_cells (find_cell_idx,
 * pp_gpu.cl:834-867, as a full offset table). */
int pp_cell_offsets_host(uint32_t n, const uint32_t *sorted_keys,
	uint32_t n_cells, uint32_t *off);

/* ------------------------------------------------------------------ */
/* Batched runs: many independent replications in one launch per step. */
/* ------------------------------------------------------------------ */

typedef struct pp_run_desc {
	PPParameters params;   /* params.iters = iterations of this run */
	uint64_t seed;
} pp_run_desc;

/* Called from pp_batch_run after the run's last iteration with its
 * params.iters + 1 stats rows. */
typedef void (*pp_stats_cb)(int run, const PPStatistics *rows,
	uint32_t n_rows, void *user);

typedef struct pp_batch_opts {
	int device;
	uint32_t pool_factor;   /* agent pool = pool_factor x initial agents (default 4) */
	uint32_t tile_cells;    /* 0 = autotune */
	uint32_t sort_digit_bits; /* 0 = autotune */
	uint32_t use_graph;     /* 1 = CUDA graph per iteration */
	uint32_t stats_chunk;   /* iterations between stats copies to the host */
	uint32_t autotune;      /* 1 = when tile_cells is 0, tune on the largest
	                           run's parameters at the batch's pool density */
	uint32_t agent_size;    /* energy field of every run, as pp_opts.agent_size */
} pp_batch_opts;

void pp_batch_opts_default(pp_batch_opts *opts);

/* Run `n_runs` independent simulations to completion in one shared state:
 * every kernel launch covers all runs. Each run's stats equal those of the
 * same run alone. */
int pp_batch_run(const pp_run_desc *runs, int n_runs,
	const pp_batch_opts *opts, pp_stats_cb cb, void *user);

/* ------------------------------------------------------------------ */
/* Serving: continuous batching of arriving runs.                      */
/* ------------------------------------------------------------------ */

typedef struct pp_server pp_server;

typedef struct pp_serve_opts {
	int device;
	uint64_t mem_budget_bytes;  /* device memory cap for resident runs   */
	uint32_t max_runs;          /* resident-run slots                     */
	uint32_t pool_factor;       /* agent slots per run = factor x initial */
	uint32_t stats_chunk;       /* iterations between stats streaming     */
	uint32_t ss_from;           /* focal measures' steady state: t > ss_from */
	uint32_t agent_size;        /* energy field of every run, as pp_opts.agent_size */
	uint32_t tile_cells;        /* cells per tile: 512, 1024 or 2048 (0 = default, 2048) */
} pp_serve_opts;

void pp_serve_opts_default(pp_serve_opts *opts);

int pp_serve_create(const pp_serve_opts *opts, pp_server **out);

/* Queue a run; it is admitted when slots and memory allow. `id` receives
 * a request id. */
int pp_serve_submit(pp_server *srv, const pp_run_desc *run, uint64_t *id);

/* Cancel a queued or resident request. */
int pp_serve_cancel(pp_server *srv, uint64_t id);

/* Advance every resident run by up to `n_iters` iterations (one shared
 * launch sequence per iteration), admitting queued runs first. */
int pp_serve_poll(pp_server *srv, uint32_t n_iters);

typedef struct pp_serve_event {
	uint64_t id;
	int status;          /* PP_SUCCESS, PP_OUT_OF_RESOURCES, PP_ERR_CANCELLED */
	uint32_t n_rows;     /* rows delivered so far for this request       */
	uint32_t done;       /* 1 when the run has finished                  */
} pp_serve_event;

/* Copy rows [first, first + n) of request `id`'s stats (available rows
 * only); `n_out` receives the number copied. */
int pp_serve_read(pp_server *srv, uint64_t id, uint32_t first, uint32_t n,
	PPStatistics *rows, uint32_t *n_out);

/* Status of request `id`. */
int pp_serve_status(pp_server *srv, uint64_t id, pp_serve_event *ev);

/* Number of queued and resident runs. */
int pp_serve_load(pp_server *srv, uint32_t *queued, uint32_t *resident);

/* Ids of requests that finished (completed, failed or cancelled) since the
 * last call, oldest first: up to `max` into ids, their number in *n_out.
 * Lets a client poll without a status call per pending request. */
int pp_serve_finished(pp_server *srv, uint64_t *ids, uint32_t max,
	uint32_t *n_out);

/* The focal measures of a finished request (PP_INVALID_ARGS until it has
 * finished successfully). */
int pp_serve_focal(pp_server *srv, uint64_t id, pp_focal *out);

/* Release a finished request's stats. */
int pp_serve_release(pp_server *srv, uint64_t id);

int pp_serve_destroy(pp_server *srv);

/* ------------------------------------------------------------------ */
/* Autotuning (no counterpart in the reference, which takes its work   */
/* sizes from command-line options: pp_gpu.c:310-410).                */
/* ------------------------------------------------------------------ */

typedef struct pp_tuning {
	uint32_t tile_cells;        /* cells per act tile                      */
	uint32_t sort_pipeline;     /* 1 = sort pipeline, 0 = fused            */
	uint32_t sort_digit_bits;   /* 0 = the library's choice                */
	float ns_per_agent_step;    /* measured device cost of the winner      */
} pp_tuning;

/* Measure the candidate geometries (fused pipeline on tiles of 512..8192
 * cells, sort pipeline on 1024..8192) on a sample of the workload -- the
 * same parameters on at
 * most 4096 x 4096 cells with agents and pool scaled by area -- and return
 * the one with the lowest device time per agent-step. Results are cached
 * per device and workload shape (and in the file named by PP_TUNE_CACHE,
 * if set). `max_agents` is the pool the real run will use (0 = default). */
int pp_autotune(const PPParameters *params, uint64_t seed, uint32_t max_agents,
	int device, pp_tuning *out);

/* The tuning pp_batch_run uses when opts->autotune is set: pp_autotune on
 * the batch's largest run at the batch's pool density. */
int pp_batch_autotune(const pp_run_desc *runs, int n_runs,
	const pp_batch_opts *opts, pp_tuning *out);

/* Library version string. */
const char *pp_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PPHPC_GB300_H */
