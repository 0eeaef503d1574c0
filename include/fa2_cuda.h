/*
 * fa2_cuda.h -- entry points of libfa2cuda.so beyond the package's fa2.h.
 *
 * fa2.h holds the interface the package's C code links against; these add a
 * device-resident layout session (the state of fa2_full_run kept on the GPU
 * between calls), per-step forces for parity checks, phase timings and tree
 * introspection. They follow fa2.h's conventions: 0 = success, a message in
 * fa2_gpu_error() otherwise, every pointer owned by the caller, positions and
 * forces as x[0..n) then y[0..n).
 */
#ifndef FA2_CUDA_H
#define FA2_CUDA_H

#include <stdint.h>

#include "fa2.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fa2cu_layout fa2cu_layout;

/* How a resident layout computes the repulsion. */
enum {
    FA2CU_REPULSION_BH = 0,    /* Barnes-Hut over the Morton/Karras tree,
                                  as fa2_full_run (no counterpart: the
                                  reference's src/gpu_full.c:403-499 loop) */
    FA2CU_REPULSION_EXACT = 1  /* every pair, as src/forceatlas2.c:278-294 */
};

/* Upload the graph and the start positions of fa2_full_params once and keep
 * the layout on the device (positions, forces, tree, FP64 speed state).
 * p->iterations, p->profile and p->interrupted are not used here. NULL on
 * error. No reference counterpart: src/gpu_full.c:164-396 inlined in
 * fa2_full_run. */
fa2cu_layout *fa2cu_layout_open(const fa2_full_params *p, const double *pos,
                                int repulsion);

/* Enqueue `iterations` iterations on the layout's stream; returns without
 * waiting. The speed update runs on the device: no host round trip. */
int fa2cu_layout_iterate(fa2cu_layout *L, int iterations);

/* Wait for the layout's stream. Returns non-zero with the message of
 * fa2_full_run (src/gpu_full.c:486-491) if the totals became invalid. */
int fa2cu_layout_sync(fa2cu_layout *L);

/* Download / replace the positions (x then y, doubles). */
int fa2cu_layout_positions(fa2cu_layout *L, double *pos);
int fa2cu_layout_set_positions(fa2cu_layout *L, const double *pos);

/* Forces of one iteration at positions pos (repulsion, gravity, attraction),
 * into f (x then y), added up as the layout's iteration adds them (single
 * precision Barnes-Hut with the "overlap" option: the repulsion plus the
 * sum of gravity and attraction; otherwise the reference's order). The
 * layout's positions are replaced by pos. */
int fa2cu_layout_forces(fa2cu_layout *L, const double *pos, double *f);

/* Speed, speed efficiency and the last swing / traction totals (FP64). */
int fa2cu_layout_speed(fa2cu_layout *L, double state[4]);

/* The layout's CUDA stream (a cudaStream_t), for timing with events. */
void *fa2cu_layout_stream(fa2cu_layout *L);

/* Run `iterations` iterations phase by phase with CUDA events between the
 * phases, adding the milliseconds of each to ms[FA2_FULL_NTIMES] (slots of
 * FA2_FULL_T_*; ms[FA2_FULL_T_TOTAL] gets the sum). */
int fa2cu_layout_phase_times(fa2cu_layout *L, int iterations, double *ms);

/* The Karras construction at positions pos: Morton keys and node order
 * (sorted), child / range (2(n-1)), parent (2n-1), and per internal node
 * (cx, cy, m, size^2) in ni (4(n-1)). Barnes-Hut layouts only. */
int fa2cu_layout_tree(fa2cu_layout *L, const double *pos, uint32_t *key,
                      uint32_t *order, int *child, int *range, int *parent,
                      double *ni);

/* Tree nodes visited and node pairs computed by one Barnes-Hut traversal at
 * the current positions (an instrumented, untimed variant). */
int fa2cu_layout_traversal_counts(fa2cu_layout *L, double counts[2]);

/* Set a tuning option of the layout (nonzero and a message for an unknown
 * name or value). Every walk computes the same interactions; walks 0-4 add
 * them up in the same order (identical forces), walk 5 in another (forces
 * equal to ~1e-7 in single precision):
 *   "walk"         Barnes-Hut walk: 1 one independent walk per thread
 *                  (default in double precision), 0 warp-synchronous (lanes
 *                  walk together, keeping their own decisions), 2 the
 *                  per-thread walk compiled without its register bound, 3 /
 *                  4 two / four Morton neighbours per thread, 5 one walk per
 *                  thread visiting regions only, its node pairs queued and
 *                  summed after the far regions (default in single
 *                  precision);
 *   "climb"        leaves per thread of the bottom-up sums: 1, 2, 4 or 8
 *                  contiguous, -2 or -4 interleaved over the warp (default:
 *                  1 below one wave of threads, else 2 in float, 4 in
 *                  double);
 *   "sort_threads" 256, 512 or 1024 threads per sort tile (default: 512
 *                  below 600000 nodes, else 1024);
 *   "sort_block"   1: the one-block sort (at most 4096 nodes; default there),
 *                  0: the tiled sort;
 *   "keep_traction" 1: keep each node's traction of the last iteration for
 *                  fa2cu_layout_swing (n more reals on the device);
 *   "overlap"      single precision, Barnes-Hut: 1 gravity and attraction
 *                  computed on a second stream beside the tree build and
 *                  the walk (forked after the sort; default), into a buffer
 *                  of their own that is then added to the repulsion; 2 the
 *                  same forked after the tree build; 0 the attraction after
 *                  the walk, added to the repulsion node by node (forces
 *                  equal to ~1e-7);
 *   "attract_grid" blocks per SM of that attraction, 1 (default) to 8;
 *   "join_blocks"  blocks of 256 threads of the join that adds it to the
 *                  repulsion and sums the swing totals (default 608: few
 *                  block partials for its last block);
 *   "pdl"          1: the iteration's kernels on the main stream launched
 *                  as programmatic dependents (each is scheduled as its
 *                  predecessor finishes; default below 500,000 nodes), 0:
 *                  ordinary launches (identical results). */
int fa2cu_layout_option(fa2cu_layout *L, const char *name, double value);

/* A figure of the layout, by name: "launches_per_iteration" (kernels of one
 * captured iteration), "heavy_nodes" (nodes of 128 incidences or more, whose
 * attraction a warp each sums in single precision), "nodes", "incidences".
 * -1 with a message for an unknown name. */
double fa2cu_layout_info(fa2cu_layout *L, const char *name);

/* Each node's swinging (sw, n doubles) and traction (tr, n doubles; needs
 * the option keep_traction, else pass NULL) of the last iteration, the
 * values the swing/traction totals of fa2cu_layout_speed sum (fixed nodes
 * excluded). Either pointer may be NULL. */
int fa2cu_layout_swing(fa2cu_layout *L, double *sw, double *tr);

/* Bytes of device memory held by the layout. */
double fa2cu_layout_bytes(const fa2cu_layout *L);

void fa2cu_layout_close(fa2cu_layout *L);

/* ---- graphs given as edge lists ---------------------------------------- */

/* The preparation C_forceatlas2_large does on the host before fa2_full_run
 * (reference src/forceatlas2.c:868-902), on the device: mass = 1 + degree
 * (a self-loop counts twice), the symmetric incidence lists with each node's
 * incidences in edge order (self-loops have none), coefficient
 * coef * w[e] (/ mass[from[e]] when outbound, coef = the mean mass; else
 * coef = 1). from / to: m edges, 0-based; w: m weights (after the R layer's
 * weight transformations). Outputs on the host: mass[n], inc_off[n + 1],
 * inc_node and inc_coef (at most 2m). Returns the number of incidences, or -1
 * with a message ("edge %d refers to a node that does not exist", the first
 * such edge numbered from 1, as the reference). No reference counterpart as
 * a separate call. */
long long fa2cu_graph_prep(int device, int n, int m, const int *from,
                           const int *to, const double *w, int outbound,
                           double *mass, int *inc_off, int *inc_node,
                           double *inc_coef);

/* fa2cu_layout_open with the graph given as its edge list, prepared on the
 * device as fa2cu_graph_prep (p's inc_off, inc_node, inc_coef and mass are
 * not read). */
fa2cu_layout *fa2cu_layout_open_edges(const fa2_full_params *p, int m,
                                      const int *from, const int *to,
                                      const double *w, int outbound,
                                      const double *pos, int repulsion);

/* fa2_full_run with the graph given as its edge list (C_forceatlas2_large's
 * host preparation moved to the device); the same results bit for bit. */
int fa2cu_full_run_edges(const fa2_full_params *p, int m, const int *from,
                         const int *to, const double *w, int outbound,
                         double *pos, double *times);

/* ---- batched layouts --------------------------------------------------- */

typedef struct fa2cu_batch fa2cu_batch;

/* Lay out `count` independent graphs together, every one of them by one
 * thread block of a persistent launch (no reference counterpart: the
 * reference lays out one graph per call). graphs[g] describes graph g
 * (n >= 1) with its own settings as for fa2_full_run; pos[g] holds its start
 * positions (x then y). Device and precision are those of graphs[0].
 * Graphs with fewer than exact_below nodes use the exact repulsion, the others
 * Barnes-Hut over their own Morton/Karras tree; threads is the block size
 * (256 or 512); nodes_per_thread (1 or 2) the tile shape of the exact sum
 * (each thread sums that many nodes against the block's tile of `threads`
 * records in shared memory). exact_below < 0, threads == 0 or
 * nodes_per_thread == 0: the values measured by fa2cu_batch_tune on this
 * device. A graph's result does not depend on the other graphs of the batch
 * (nor on the tile shape). NULL on error. */
fa2cu_batch *fa2cu_batch_open(const fa2_full_params *graphs, int count,
                              const double *const *pos, int exact_below,
                              int threads, int nodes_per_thread);
/* Enqueue `iterations` iterations of every graph (one launch). */
int fa2cu_batch_iterate(fa2cu_batch *B, int iterations);
int fa2cu_batch_sync(fa2cu_batch *B);
/* Positions of graph g (x then y). */
int fa2cu_batch_positions(fa2cu_batch *B, int g, double *pos);
/* Forces of graph g in the last iteration, at the positions before its
 * displacement (fx then fy); after a sync. */
int fa2cu_batch_forces(fa2cu_batch *B, int g, double *f);
/* Speed, efficiency and last swing / traction totals of graph g. */
int fa2cu_batch_speed(fa2cu_batch *B, int g, double state[4]);
void *fa2cu_batch_stream(fa2cu_batch *B);
/* Run `iterations` iterations of every graph with a clock read after each
 * phase (an uncaptured, instrumented launch) and return the SM cycles spent
 * per phase, summed over the blocks: codes (bounding box, Morton), sort,
 * tree (gather, Karras), sums (bottom-up), repulsion, attraction, totals
 * (swing, traction, speed), move. */
int fa2cu_batch_phase_cycles(fa2cu_batch *B, int iterations, double cycles[8]);
double fa2cu_batch_bytes(const fa2cu_batch *B);
void fa2cu_batch_close(fa2cu_batch *B);

/* The autotuner: exact-vs-Barnes-Hut crossover (in nodes), block size and
 * the exact sum's nodes per thread of the batched engine, measured on
 * `device` in the given precision (timed batches of Erdos-Renyi graphs of 64
 * to 16384 nodes). Cached per device and precision for the process.
 * nodes_per_thread may be NULL. */
int fa2cu_batch_tune(int device, int use_double, int *exact_below,
                     int *threads, int *nodes_per_thread);

/* ---- serving ------------------------------------------------------------ */

/* A layout server (no reference counterpart: the reference runs one layout
 * per call, start to end). Jobs are submitted from any host thread; an
 * admission thread makes each one resident on the device (graph, positions,
 * tree buffers and speed state, in a memory pool of the server) while the
 * estimated device footprint of the resident jobs stays within the budget
 * and fewer than max_jobs are resident; a scheduling thread interleaves the
 * jobs' iterations, `chunk` at a time, each job on a stream of its own
 * whose priority rises as its work (nodes x iterations) falls. Jobs are
 * admitted in arrival order, or least work first. A job's result is the
 * same as the single-layout path's for its inputs, whatever else runs beside
 * it. */
typedef struct fa2cu_server fa2cu_server;

typedef struct {
    int device;
    double hbm_budget; /* bytes the resident jobs may hold; <= 0: 80 % of the
                          device's free memory at open */
    int max_jobs;      /* jobs resident at once; <= 0: 16 */
    int chunk;         /* iterations enqueued per job at a time; <= 0: 16 */
    int policy;        /* admission order: FA2CU_ADMIT_ARRIVAL (0) or
                          FA2CU_ADMIT_LEAST_WORK (1: the queued job of least
                          nodes x iterations first) */
} fa2cu_server_config;

enum { FA2CU_ADMIT_ARRIVAL = 0, FA2CU_ADMIT_LEAST_WORK = 1 };

fa2cu_server *fa2cu_server_open(const fa2cu_server_config *cfg);

/* Submit a layout job: the graph and settings as for fa2_full_run (its
 * p->iterations iterations in p->use_double precision; p->device, profile,
 * source and interrupted are ignored), start positions pos (x then y),
 * repulsion FA2CU_REPULSION_BH or FA2CU_REPULSION_EXACT. Everything is
 * copied before the call returns. Returns the job's id (>= 0), or -1 with a
 * message (invalid job, or a footprint above the whole budget). */
long long fa2cu_server_submit(fa2cu_server *S, const fa2_full_params *p,
                              const double *pos, int repulsion);

/* Wait up to timeout_s seconds (< 0: no limit) for job `id` to end, or for
 * any ended job not yet claimed if id < 0, and claim it. info[8]: submit,
 * resident and end times (fa2_now's clock), status (0 done, 1 failed), n,
 * iterations, footprint bytes, final speed. Returns the id, -1 on timeout,
 * -2 if there is no such job (or, for id < 0, none left to claim). */
long long fa2cu_server_wait(fa2cu_server *S, long long id, double timeout_s,
                            double info[8]);

/* Copy an ended job's final positions into pos (2n doubles, x then y; may be
 * NULL) and release the job. 0, or 1 with a message: the job has not ended
 * (or was collected), or it failed (its own message). */
int fa2cu_server_collect(fa2cu_server *S, long long id, double *pos);

/* out[8]: jobs queued, resident, done, failed; footprint bytes resident now
 * and at most so far; the budget; device bytes reserved by the pool. */
int fa2cu_server_stats(fa2cu_server *S, double out[8]);

/* Stop the threads, drop the jobs not collected, release the pool. */
void fa2cu_server_close(fa2cu_server *S);

/* Device bytes a layout of n nodes and ninc incidences holds on the current
 * device (its buffers and the staging of the graph upload): the server's
 * admission estimate. */
double fa2cu_layout_footprint(int n, int ninc, int adjust, int any_fixed,
                              int use_double, int repulsion);

/* Morton codes and stable Morton order of n nodes whose positions are
 * already on the device, without allocating any memory: the one entry point
 * for callers that cannot call cudaMalloc (their device memory belongs to
 * another allocator, or they cannot afford an allocation's synchronisation
 * or failure once started). It has no counterpart in the reference.
 *   pos    device, n interleaved (x, y) floats;
 *   key    device, n uint32: the sorted Morton codes (16 bits per axis);
 *   order  device, n uint32: node indices in Morton order, ties by index;
 *   stream the cudaStream_t to run on (NULL: the default stream).
 * 1 <= n <= 2^20, larger n is an error. pos must be 8-byte aligned, key and
 * order 4-byte aligned (refused otherwise). Its scratch is a static device
 * array of the library (about 9 MB per GPU, held until exit) shared by every
 * call: calls that overlap on the GPU race. The first call on a device looks
 * the array up on that device, which (with CUDA's lazy module loading) also
 * loads the library's device code and the array there and may allocate and
 * synchronise: make it up front (fa2cu_noalloc_status does only that
 * lookup), before any stream capture. Returns 0 once the work is queued, or
 * non-zero with a message for fa2_gpu_error(). */
int fa2cu_morton_order_noalloc(int n, const float *pos, uint32_t *key,
                               uint32_t *order, void *stream);

/* Companion of fa2cu_morton_order_noalloc, on the current device: waits for
 * `stream`, then returns 0 if the last call there completed, or non-zero
 * with a message if one of its sort's bounded waits gave up (its key and
 * order are then wrong). Also the up-front set-up of the scratch array. It
 * allocates nothing. No counterpart in the reference. */
int fa2cu_noalloc_status(void *stream);

/* Library build description (compile flags and architecture). */
const char *fa2cu_build_info(void);

#ifdef __cplusplus
}
#endif

#endif
