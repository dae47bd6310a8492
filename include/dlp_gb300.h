/*
 * dlp_gb300.h - C ABI of the GB300-native DynLP per-batch update path.
 *
 * Plain pointers and sizes only. Every entry point returns a status code
 * (DLP_OK on success) instead of exiting; dlp_last_error() holds a message for
 * the calling thread's last failure. Device pointers are CUDA device
 * addresses on the current device; `stream` is a cudaStream_t passed as void*
 * (NULL = the legacy default stream).
 *
 * Groups of entry points:
 *   1. input generation (host only),
 *   2. a resident session that keeps one dynamic graph on the GPU and applies
 *      batches with no host round trip inside a batch;
 *   2b. the batch engine: many resident graphs, one persistent launch per
 *      step over all of them, snapshot/restore, and the autotuner;
 *   2c. continuous batching: sliced steps and the request server;
 *   3. the reference's five step launchers on caller-owned device arrays in the
 *      reference's layout (drop-in for src/sparsifySubgraph.cu,
 *      src/connectedComponents.cu, src/labelInitialization.cu,
 *      src/iterativePropagation.cu of SMShovan/LabelPropCUDA), IrLP, and an
 *      allocation-free propagation entry point;
 *   4. device helpers (malloc/free/copies) for callers without a CUDA runtime.
 * The C++ shims in dynLP.h, sparsifySubgraph.h, connectedComponents.h,
 * labelInitialization.h and iterativePropagation.h call these.
 */
#ifndef DLP_GB300_H
#define DLP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DLP_ABI_VERSION 1

enum dlp_status {
  DLP_OK = 0,
  DLP_ERR_INVALID_ARGUMENT = 1, /* bad size, null pointer, vertex id out of range */
  DLP_ERR_CUDA = 2,             /* a CUDA runtime call failed */
  DLP_ERR_OUT_OF_MEMORY = 3,
  DLP_ERR_TIMEOUT = 4,          /* a device-side wait ran past its limit */
  DLP_ERR_NO_DEVICE = 5,        /* no usable sm_103 GPU */
  DLP_ERR_NOT_CONVERGED = 6,    /* connected components exceeded the round cap */
  DLP_ERR_INTERNAL = 7
};

enum dlp_semantics {
  DLP_SEMANTICS_REF = 0,  /* the reference's behaviour (default) */
  DLP_SEMANTICS_SPEC = 1  /* the documented intent: full affected set, permanent deletions */
};

int dlp_abi_version(void);
const char *dlp_status_string(int status);
/* Message of the calling thread's last failed call ("" if none). */
const char *dlp_last_error(void);

/* ------------------------------------------------------------------------ */
/* 1. Input generation (host). Replaces generateSparseGraph                  */
/*    (src/generateSparseGraph.cu:118) and generateBatches                   */
/*    (src/generateBatches.cu:44) with the same seeded output.               */
/* ------------------------------------------------------------------------ */

typedef struct dlp_problem dlp_problem;

/* A batch as plain arrays (host or device pointers, depending on the call). */
typedef struct dlp_batch_view {
  const int *inserted;       /* vertices that arrive in this batch */
  int num_inserted;
  const int *gt_ids;         /* subset of inserted with ground-truth labels */
  const float *gt_labels;    /* 0.0 / 1.0 */
  int num_gt;
  const int *deleted;        /* vertices removed in this batch */
  int num_deleted;
  const int *edge_src;       /* edges that become live in this batch (src < dst) */
  const int *edge_dst;
  const float *edge_weight;
  int num_edges;
} dlp_batch_view;

int dlp_problem_generate(int num_nodes, int avg_degree, int num_batches, unsigned seed,
                         float gt_fraction, float deleted_fraction, dlp_problem **out);
void dlp_problem_free(dlp_problem *p);
int dlp_problem_num_nodes(const dlp_problem *p);
int64_t dlp_problem_num_edges(const dlp_problem *p);
int dlp_problem_num_batches(const dlp_problem *p);
const int *dlp_problem_row_ptr(const dlp_problem *p);
const int *dlp_problem_col_ind(const dlp_problem *p);
const float *dlp_problem_values(const dlp_problem *p);
const float *dlp_problem_true_labels(const dlp_problem *p);
/* Host views into the problem's storage (valid until dlp_problem_free). */
int dlp_problem_batch(const dlp_problem *p, int batch, dlp_batch_view *out);
/* <prefix>RowPtr.txt, ColInd.txt, Values.txt, TrueLabels.txt in the reference's
 * text format (src/generateSparseGraph.cu:224-271). */
int dlp_problem_write_csr(const dlp_problem *p, const char *prefix);
/* Binary input cache. The reference regenerates its input on every run and
 * writes its graph only as text it never reads back
 * (src/generateSparseGraph.cu:218-274); these keep a generated problem in one
 * binary file keyed by the generator arguments.
 * dlp_problem_save writes p to path (a temporary file, then a rename).
 * dlp_problem_load reads a file written by dlp_problem_save; a file whose
 * recorded size or payload hash does not match is refused.
 * dlp_problem_generate_cached reads the file of these arguments from
 * cache_dir when it is present and valid, else generates the problem (same
 * output as dlp_problem_generate) and (re)writes the file (cache_dir is
 * created when missing; its parent must exist); *from_cache (may be NULL) is
 * 1 when the problem came from the file. */
int dlp_problem_save(const dlp_problem *p, const char *path);
int dlp_problem_load(const char *path, dlp_problem **out);
int dlp_problem_generate_cached(int num_nodes, int avg_degree, int num_batches, unsigned seed,
                                float gt_fraction, float deleted_fraction, const char *cache_dir,
                                dlp_problem **out, int *from_cache);
/* Mean weight of the non-deleted edges of a CSR (auto tau, src/dynLP.cu:90-102). */
float dlp_mean_edge_weight(int64_t num_edges, const int *col_ind, const float *values);

/* ------------------------------------------------------------------------ */
/* 2. Resident session: one dynamic graph on the GPU                          */
/*    (the per-batch loop of runDynLP, src/dynLP.cu:284-558).                 */
/* ------------------------------------------------------------------------ */

/* Division in the label updates (propagation and initialisation). IEEE
 * round-to-nearest is the default and what the CPU oracle computes, bit for
 * bit. The reference is built with --use_fast_math (Makefile:52), whose `/` is
 * the CUDA fast division; DLP_ARITH_REFERENCE_FAST_MATH uses that division
 * too, for results that follow the reference's own binary more closely (its
 * float-atomic supernode sums still add in a varying order). */
enum dlp_arithmetic { DLP_ARITH_IEEE = 0, DLP_ARITH_REFERENCE_FAST_MATH = 1 };
/* The same choice for the reference-layout step launchers below
 * (dlp_label_initialization, dlp_iterative_propagation and its allocation-free
 * variant) launched afterwards by this process. */
int dlp_set_launcher_arithmetic(int arithmetic);

typedef struct dlp_config {
  float tau;             /* sparsification threshold; < 0: mean full-graph edge weight */
  float delta;           /* convergence threshold (> 0) */
  int max_iterations;    /* propagation pass cap */
  int semantics;         /* enum dlp_semantics */
  int device;            /* CUDA device ordinal */
  int record;            /* nonzero: keep per-batch artefacts for dlp_session_artefact */
  int narrow_lanes;      /* lanes per short row in full-grid propagation passes: 4, 8,
                            16 or 32; or 1: one lane per row of at most 8 entries
                            (32 rows in flight per warp) and 4-lane groups for rows
                            of 9 to 32; 0 = 8 (dlp_autotune picks one for a
                            workload); same results */
  int blocks_per_sm;     /* persistent grid occupancy; 0 = from the occupancy query */
  double wait_timeout_s; /* limit for any device-side wait; <= 0: 2 s */
  int small_frontier_solo; /* bit 0: passes over small frontiers run on one
                              thread block with block barriers; bit 1: passes
                              over mid-size frontiers run on a sub-grid with its
                              own barrier; bit 2: within the one-block mode,
                              frontiers of at most 64 loaded rows run on 8 warps
                              with a named barrier. Default 7 (all); same
                              results. */
  int solo_entry;        /* one-block mode for total frontiers of at most this
                            many vertices; 0 = 512, at most 1024 (autotuned) */
  int subgrid_entry;     /* sub-grid mode for total frontiers of at most this
                            many; 0 = 2048, at most 4096 (autotuned) */
  int arithmetic;        /* enum dlp_arithmetic: the division of the label
                            updates (default DLP_ARITH_IEEE) */
} dlp_config;

void dlp_config_default(dlp_config *cfg);

/* Per-batch results. */
typedef struct dlp_batch_stats {
  int batch;
  int iterations;          /* propagation passes (iterationsUsed) */
  int num_components;      /* connected components among inserted vertices */
  int num_sub_edges;       /* 2 x new-new edges with w > tau (numSubEdges) */
  int hook_edges;          /* edges hooked by the components step */
  int hook_rounds;         /* hook passes until no change; hooks of one pass race (as in the
                              reference), so this count can vary from run to run while the
                              components themselves do not */
  int seed_frontier;       /* |F_0| */
  int seed_marks;          /* vertices marked affected before filtering */
  int64_t affected_edges;  /* sum over passes of the frontier's row lengths */
  int64_t frontier_visits; /* sum over passes of the frontier size */
  int64_t correct;         /* active non-GT vertices on the right side of 0.5 */
  int64_t total;           /* active non-GT vertices */
  float accuracy;          /* correct / total (1 when total == 0) */
  int status;              /* DLP_OK or the device-reported error */
  int init_branch;         /* 0 none, 1 component init, 2 no-edge init */
  int hook_truncated;      /* ref: num_sub_edges exceeded the batch's edge count */
  float device_ms;         /* device time of the batch kernel */
  int dirty_rows;          /* live rows rebuilt (changed vertices and their neighbours) */
  int64_t dirty_entries;   /* full-graph entries read by that rebuild */
} dlp_batch_stats;

typedef struct dlp_session dlp_session;

/* Uploads the full graph (host CSR, int32 rows sorted by column) and creates the
 * resident state. true_labels (may be NULL) feeds the accuracy counters.
 * vertex_batch_map (may be NULL) gives the batch in which each vertex arrives
 * (-1: never); with it a vertex is live in batch b only if it arrived by b, as
 * the reference's host rebuild requires (src/dynLP.cu:143-145). */
int dlp_session_create(const dlp_config *cfg, int num_nodes, int64_t num_edges,
                       const int *row_ptr, const int *col_ind, const float *values,
                       const float *true_labels, const int *vertex_batch_map,
                       dlp_session **out);
int dlp_session_destroy(dlp_session *s);
/* Back to the state before the first batch (graph stays resident). */
int dlp_session_reset(dlp_session *s);
float dlp_session_tau(const dlp_session *s);
/* Applies batch `batch_index` from host arrays: copies them to the device,
 * runs the whole batch as one persistent kernel, and (if stats != NULL) waits
 * and returns the batch's statistics. */
int dlp_session_apply_batch(dlp_session *s, int batch_index, const dlp_batch_view *host_batch,
                            dlp_batch_stats *stats);
/* Same with device-resident batch arrays; never waits. */
int dlp_session_apply_batch_device(dlp_session *s, int batch_index,
                                   const dlp_batch_view *device_batch);
/* Waits for queued batches; then dlp_session_stats returns any batch's numbers. */
int dlp_session_synchronize(dlp_session *s);
int dlp_session_stats(dlp_session *s, int batch_index, dlp_batch_stats *out);
int dlp_session_read_labels(dlp_session *s, float *host_labels);
void *dlp_session_stream(dlp_session *s);
/* Device time from the start of the latest application of batch `first` to the
 * end of the latest application of batch `last` (CUDA events on the session
 * stream); waits for the stream. */
int dlp_session_elapsed_ms(dlp_session *s, int first, int last, float *ms);
/* Device-side diagnostics after a failed batch (see dlp_engine_debug). */
int dlp_session_debug(dlp_session *s, int *out4);

/* Artefacts of the last applied batch when cfg.record != 0 (4-byte elements;
 * *count receives the element count; host_out may be NULL to query it). */
enum dlp_artefact {
  DLP_ART_SEED_MARKS = 0,   /* int32 ascending */
  DLP_ART_FRONTIER0 = 1,    /* int32 ascending */
  DLP_ART_SUB_EDGES = 2,    /* int32 pairs (u,v),(v,u) in raw edge order */
  DLP_ART_COMP_ROOT = 3,    /* int32 per inserted vertex: min vertex id of its component, -1 */
  DLP_ART_INIT_LABELS = 5,  /* fp32 per inserted vertex */
  DLP_ART_FRONTIER_SIZES = 6,
  DLP_ART_ROW_LENGTHS = 7,  /* int32 per vertex: live row length (before soft delete) */
  DLP_ART_LABELS = 10
};
int dlp_session_artefact(dlp_session *s, int which, void *host_out, int64_t capacity,
                         int64_t *count);

/* ------------------------------------------------------------------------ */
/* 2b. Batch engine: many resident graphs; one step applies one batch to     */
/*     each of several graphs in ONE cooperative launch (flattened work      */
/*     lists, per-graph convergence). A session is a one-graph engine.       */
/* ------------------------------------------------------------------------ */

typedef struct dlp_engine dlp_engine;

/* max_graphs <= 1024; memory_budget_bytes = 0 means no budget. */
int dlp_engine_create(const dlp_config *cfg, int max_graphs, size_t memory_budget_bytes, dlp_engine **out);
int dlp_engine_destroy(dlp_engine *e);
/* Device bytes a graph of this size occupies once added (admission). */
size_t dlp_engine_graph_bytes(int num_nodes, int64_t num_edges, int with_truth, int with_batch_map, int record);
size_t dlp_engine_bytes_in_use(const dlp_engine *e);
/* Uploads a graph (same arrays as dlp_session_create); fails with
 * DLP_ERR_OUT_OF_MEMORY when it would exceed the budget. */
int dlp_engine_add_graph(dlp_engine *e, int num_nodes, int64_t num_edges, const int *row_ptr,
                         const int *col_ind, const float *values, const float *true_labels,
                         const int *vertex_batch_map, int *graph_id);
/* Frees a graph's device memory (eviction); its id becomes free. */
int dlp_engine_remove_graph(dlp_engine *e, int graph_id);
/* Copies a graph's whole device state (graph, labels, live rows, counters,
 * the statistics kept so far) to host memory, so that it can be evicted with
 * dlp_engine_remove_graph and brought back later by dlp_engine_restore with
 * identical results. With out == NULL, *bytes receives the size needed. Not
 * allowed while the graph's batch is in progress. No counterpart in the
 * reference (its graph state lives in its driver loop only). */
int dlp_engine_snapshot(dlp_engine *e, int graph_id, void *out, size_t capacity, size_t *bytes);
/* Makes a snapshotted graph resident again, in this or another engine with
 * the same record flag and semantics; counts against the memory budget like
 * dlp_engine_add_graph. *graph_id receives its (possibly new) id. */
int dlp_engine_restore(dlp_engine *e, const void *snapshot, size_t bytes, int *graph_id);
/* Same, into the given free graph id (so a graph can keep its id across an
 * eviction). */
int dlp_engine_restore_as(dlp_engine *e, const void *snapshot, size_t bytes, int graph_id);
/* Keeps a free graph id for a graph that was removed to host memory:
 * dlp_engine_add_graph and dlp_engine_restore skip a held id, and
 * dlp_engine_restore_as into it releases the hold. Release without a restore
 * with dlp_engine_release_id. No counterpart in the reference. */
int dlp_engine_hold_id(dlp_engine *e, int graph_id);
int dlp_engine_release_id(dlp_engine *e, int graph_id);
/* Device bytes a resident graph occupies (0 for an unknown id). */
size_t dlp_engine_graph_resident_bytes(const dlp_engine *e, int graph_id);
int dlp_engine_reset_graph(dlp_engine *e, int graph_id);
float dlp_engine_tau(const dlp_engine *e, int graph_id);
void *dlp_engine_stream(dlp_engine *e);
/* One step over `count` distinct graphs: batch i (host arrays) is applied to
 * graph_ids[i] as its batch batch_indices[i]. With stats != NULL the call
 * waits and fills stats[i]. */
int dlp_engine_step(dlp_engine *e, int count, const int *graph_ids, const int *batch_indices,
                    const dlp_batch_view *host_batches, dlp_batch_stats *stats);
/* Same with device-resident batch arrays (they need not outlive the step);
 * never waits. Neither call takes a graph whose batch is in progress in
 * sliced steps (section 2c). */
int dlp_engine_step_device(dlp_engine *e, int count, const int *graph_ids, const int *batch_indices,
                           const dlp_batch_view *device_batches);
int dlp_engine_synchronize(dlp_engine *e);
int dlp_engine_stats(dlp_engine *e, int graph_id, int batch_index, dlp_batch_stats *out);
/* Steps launched so far, and the device time from the start of step `first`
 * to the end of step `last`. */
int dlp_engine_steps(const dlp_engine *e);
/* Device-side diagnostics after a failed step: out[0] error code, out[1] last
 * phase reached (1..10), out[2] last propagation pass started, out[3] passes
 * of the last one-block / sub-grid stint. */
int dlp_engine_debug(dlp_engine *e, int *out4);
int dlp_engine_elapsed_ms(dlp_engine *e, int first_step, int last_step, float *ms);
/* Propagation passes the engine's launches have run so far, by mode, and the
 * device time they took: [0] one block (including [1]), [1] the 8-warp team
 * (passes only; its time is counted in [0]), [2] the 16-block sub-grid,
 * [3] the full grid. Diagnostics of where a workload's propagation time goes;
 * cumulative since the engine was made. */
int dlp_engine_pass_modes(dlp_engine *e, unsigned long long *passes4, double *seconds4);
int dlp_session_pass_modes(dlp_session *s, unsigned long long *passes4, double *seconds4);
int dlp_engine_read_labels(dlp_engine *e, int graph_id, float *host_labels);
int dlp_engine_artefact(dlp_engine *e, int graph_id, int which, void *host_out, int64_t capacity,
                        int64_t *count);

/* Autotuner (no counterpart in the reference, whose launch shapes are fixed).
 * Propagation sends rows of at most 32 live entries to groups of
 * narrow_lanes lanes and longer rows to whole warps, and runs each pass on one
 * block, a 16-block sub-grid or the whole grid by the size of the frontier.
 * The lane width of the short-row bucket, the two frontier thresholds
 * (solo_entry, subgrid_entry) and the persistent grid's blocks per SM are
 * chosen by timing every candidate (lanes 1/4/8 x one-block entry
 * 256/512/1024 x sub-grid entry 1024/2048/4096 x the blocks per SM the build
 * allows) on a sample the library generates with the reference generator:
 * num_graphs graphs of sizes[i] vertices and average degree degrees[i],
 * `batches` batches each, propagation capped at max_iterations passes per
 * batch for the trial. Every candidate must give identical statistics
 * (checked). The fastest is written into cfg->narrow_lanes,
 * cfg->blocks_per_sm, cfg->solo_entry and cfg->subgrid_entry; other fields are
 * kept. */
typedef struct {
  int candidates;
  int best;               /* index of the chosen candidate */
  int lanes[32];
  int blocks_per_sm[32];
  int solo_entry[32];
  int subgrid_entry[32];
  double ms[32];          /* summed device time of the sample's steps */
} dlp_tune_report;
int dlp_autotune(dlp_config *cfg, int num_graphs, const int *sizes, const int *degrees, int batches,
                 int max_iterations, dlp_tune_report *report);

/* ------------------------------------------------------------------------ */
/* 2c. Continuous batching (no counterpart in the reference, which applies   */
/*     one batch of one graph at a time). A sliced step starts new batches   */
/*     and continues unfinished ones in ONE launch, for a bounded slice of   */
/*     propagation; a server admits waiting requests between slices.         */
/* ------------------------------------------------------------------------ */

/* Starts batch batch_indices[i] on graph_ids[i] (device-resident arrays that
 * must stay valid until that batch ends) and continues every graph whose batch
 * is still in progress, in one launch. The phases before propagation always
 * complete; propagation stops after pass_budget passes (0: no limit) or once
 * slice_us microseconds have passed since the launch began (0: no limit),
 * whichever comes first. Waits for the launch. The ids of the graphs whose
 * batch ended go to finished_ids (room for max_graphs ids), their number to
 * *num_finished, the number still in progress to *num_continuing (may be
 * NULL). A graph in progress cannot start another batch; its statistics and
 * labels become readable when its batch ends. Every result is bit-identical to
 * the same batches run by unsliced steps. */
int dlp_engine_step_sliced(dlp_engine *e, int count, const int *graph_ids, const int *batch_indices,
                           const dlp_batch_view *device_batches, int pass_budget, double slice_us,
                           int *finished_ids, int *num_finished, int *num_continuing);
/* Sizes a graph's batch scratch for batches of up to max_edges new edges and
 * max_deleted deletions, so that later steps allocate nothing (scratch grows
 * on demand otherwise). */
int dlp_engine_reserve(dlp_engine *e, int graph_id, int max_edges, int max_deleted);
/* Vertex count of a resident graph, -1 for an unknown id. */
int dlp_engine_graph_nodes(const dlp_engine *e, int graph_id);
/* 1 while graph_id has a batch in progress in sliced steps, else 0. */
int dlp_engine_in_progress(const dlp_engine *e, int graph_id);

typedef struct dlp_server dlp_server;

typedef struct {
  double slice_us;            /* propagation time per step before waiting requests join (default 2000) */
  int pass_budget;            /* propagation passes per step (default 0: no limit) */
  size_t memory_budget_bytes; /* admission limit on the engine's resident bytes, the server's staging
                                 buffers and the engine scratch of running requests; idle graphs'
                                 staging buffers are freed first when a request does not fit
                                 (default 0: no limit) */
  int max_batches_per_step;   /* new batches started per step (default 0: the engine's max_graphs) */
  int serial;                 /* 1: the plain path, one request at a time run to its end (default 0) */
  int evict_idle;             /* 1: when a request does not fit the budget, graphs with no request
                                 running are evicted to host memory (least recently used first) and
                                 restored under the same id before their next request (default 0) */
} dlp_server_config;
void dlp_server_config_default(dlp_server_config *cfg);

typedef struct {
  int graph_id;               /* a graph resident in the server's engine */
  int batch_index;
  dlp_batch_view batch;       /* host arrays */
  double arrival_s;           /* dlp_server_replay only: offset from the start of the replay */
} dlp_request;

typedef struct {
  int graph_id;
  int batch_index;
  int status;                 /* DLP_OK, or why the request failed */
  double arrival_s;           /* server clock, seconds */
  double admit_s;             /* first step the batch took part in */
  double finish_s;            /* its statistics were read back */
  int steps;                  /* sliced steps the batch took part in */
  dlp_batch_stats stats;
} dlp_request_result;

/* A server drives one engine; graphs are added to the engine beforehand. */
int dlp_server_create(dlp_engine *e, const dlp_server_config *cfg, dlp_server **out);
/* Destroy a server before its engine. Graphs the server evicted to host memory
 * go back into the engine under their ids (a graph that no longer fits the
 * engine's budget is dropped and its id released). */
int dlp_server_destroy(dlp_server *s);
/* Seconds since the server was created (the clock of dlp_request_result). */
double dlp_server_clock(const dlp_server *s);
/* Sizes a graph's staging buffers and its engine scratch for requests up to
 * the given sizes, so that admission allocates nothing. */
int dlp_server_reserve(dlp_server *s, int graph_id, int max_inserted, int max_gt, int max_deleted,
                       int max_edges);
/* Queues a request (its arrays are copied); *request_id identifies it. */
int dlp_server_submit(dlp_server *s, const dlp_request *req, int *request_id);
/* One scheduling round: admits queued requests in arrival order (one batch
 * per graph at a time, within the memory budget), runs one sliced step over
 * them and the batches in progress, and writes the ids of the requests that
 * ended (up to capacity). Returns at once when nothing is queued or running. */
int dlp_server_poll(dlp_server *s, int *completed_ids, int capacity, int *num_completed);
int dlp_server_result(const dlp_server *s, int request_id, dlp_request_result *out);
/* Requests queued or running. */
int dlp_server_pending(const dlp_server *s);
/* Graphs this server evicted to host memory and restored so far. */
int dlp_server_evictions(const dlp_server *s, int *evictions, int *restores);
/* Restores graph_id if this server evicted it (evicting others if allowed and
 * needed), so that the engine's calls can reach it again. */
int dlp_server_make_resident(dlp_server *s, int graph_id);
/* Replays a trace in real time: reqs[i] (sorted by arrival_s) is submitted
 * once arrival_s seconds have passed since the call began, and the server
 * polls until every request has ended. out[i] holds request i's result with
 * times relative to the start of the replay; *makespan_s is the time until
 * the last one ended. The arrays are used in place during the call. */
int dlp_server_replay(dlp_server *s, int count, const dlp_request *reqs, dlp_request_result *out,
                      double *makespan_s);

/* ------------------------------------------------------------------------ */
/* 3. Step launchers on caller-owned device arrays, reference layout.        */
/*    Same argument meaning as the reference; they synchronise the stream    */
/*    only where a scalar result is returned through a pointer.             */
/* ------------------------------------------------------------------------ */

/* launchMarkDeletions (src/sparsifySubgraph.cu:185-203). */
int dlp_mark_deletions(int *d_row_ptr, int *d_col_ind, int *d_vertex_status, int *d_is_affected,
                       const int *d_deleted_nodes, int num_deleted, int num_nodes, void *stream);

/* launchBuildSparsifiedSubgraph (src/sparsifySubgraph.cu:205-287). The kept
 * edges are written to d_sub_col_ind / d_sub_values (destinations and weights,
 * both directions, raw edge order; each at least max(2*num_new_edges,1) long). */
int dlp_build_sparsified_subgraph(int *d_row_ptr, int *d_col_ind, float *d_values,
                                  int *d_is_affected, const int *d_vertex_status,
                                  const int *d_new_edge_src, const int *d_new_edge_dst,
                                  const float *d_new_edge_weight, int num_new_edges,
                                  const int *d_inserted_nodes, int num_inserted,
                                  const int *d_is_new_vertex, float tau, int *d_sub_row_ptr,
                                  int *d_sub_col_ind, float *d_sub_values, int *num_sub_nodes,
                                  int *num_sub_edges, void *stream);

/* launchConnectedComponents (src/connectedComponents.cu:162-290). */
int dlp_connected_components(const int *d_edge_src, const int *d_edge_dst, int num_edges,
                             const int *d_inserted_nodes, int num_inserted, int *d_component_id,
                             int *num_components, int num_nodes, void *stream);

/* launchLabelInitialization (src/labelInitialization.cu:148-187). */
int dlp_label_initialization(const int *d_row_ptr, const int *d_col_ind, const float *d_values,
                             float *d_labels, const int *d_vertex_status,
                             const int *d_component_id, int num_components,
                             const int *d_inserted_nodes, int num_inserted, const int *d_gt_class,
                             int num_nodes, void *stream);

/* launchIterativePropagation (src/iterativePropagation.cu:241-346). */
int dlp_iterative_propagation(const int *d_row_ptr, const int *d_col_ind, const float *d_values,
                              float *d_labels, float *d_labels_buffer, const int *d_vertex_status,
                              const int *d_gt_class, int *d_is_affected, int num_nodes,
                              float delta, int max_iterations, int *iterations_used,
                              void *stream);

/* Same arguments and results as dlp_iterative_propagation, but allocates no
 * device memory: its scratch is a fixed array inside this library (16 MiB +
 * 1 KiB, present on every GPU that loads the library until the process ends).
 * No counterpart in the reference, whose launchers call cudaMalloc/cudaFree on
 * every call. For callers that may not allocate device memory while running:
 * hosts that own the device's whole memory pool, or services that reserve all
 * memory up front so that nothing can fail or stall later. Limits and rules:
 * num_nodes <= 1048576 (larger graphs get DLP_ERR_INVALID_ARGUMENT); the first
 * call on a device looks up the array's address, so make it before any stream
 * capture; every call reuses the same array, so calls that overlap on the GPU
 * race and must be serialised by the caller. */
int dlp_iterative_propagation_noalloc(const int *d_row_ptr, const int *d_col_ind, const float *d_values,
                                      float *d_labels, float *d_labels_buffer, const int *d_vertex_status,
                                      const int *d_gt_class, int *d_is_affected, int num_nodes, float delta,
                                      int max_iterations, int *iterations_used, void *stream);

/* launchIrLP (src/validation.cu:145-208): full recompute of every active
 * non-ground-truth vertex per iteration until no label moves by more than
 * delta, as one cooperative launch. Result in d_labels. */
int dlp_irlp(const int *d_row_ptr, const int *d_col_ind, const float *d_values, float *d_labels,
             const int *d_vertex_status, const int *d_gt_class, int num_nodes, float delta,
             int max_iterations, int *iterations_used, void *stream);

/* ------------------------------------------------------------------------ */
/* Device helpers for bindings that have no CUDA runtime of their own.       */
/* ------------------------------------------------------------------------ */
int dlp_device_count(int *count);
/* "<name> sm_<major><minor> <SMs> SMs" of a device (the autotuner's cache key). */
int dlp_device_name(int device, char *out, int capacity);
int dlp_set_device(int device);
int dlp_malloc(void **ptr, size_t bytes);
int dlp_free(void *ptr);
int dlp_memcpy_htod(void *dst, const void *src, size_t bytes);
int dlp_memcpy_dtoh(void *dst, const void *src, size_t bytes);
int dlp_memset(void *ptr, int value, size_t bytes);
int dlp_device_synchronize(void);

#ifdef __cplusplus
}
#endif
#endif /* DLP_GB300_H */
