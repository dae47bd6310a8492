/*
 * Test infrastructure, not product code: the CPU oracle of the DynLP per-batch
 * update path (SMShovan/LabelPropCUDA). Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it, and only as the checker or the
 * timed CPU baseline; the product never calls it.
 *
 * It restates, one batch at a time, what the reference's runDynLP does
 * (src/dynLP.cu:284-558) with the same parity-relevant behaviour:
 *   - host CSR rebuild per batch                src/dynLP.cu:111-167
 *   - deletion marks and soft delete            src/sparsifySubgraph.cu:58-111
 *   - tau filter, clipped endpoint marks        src/sparsifySubgraph.cu:119-179
 *   - Shiloach-Vishkin on the raw edge prefix   src/dynLP.cu:437-440,
 *                                               src/connectedComponents.cu:162-290
 *   - supernode label initialisation            src/labelInitialization.cu:59-142
 *   - frontier propagation, stale double buffer src/iterativePropagation.cu:63-346
 *   - 0.5-threshold accuracy                    src/dynLP.cu:65-85
 * The arithmetic conventions shared with the CUDA path (summation tree,
 * explicit fmaf, IEEE division, fixed-point supernode sums, the pinned
 * convention for the reference's out-of-bounds reads) are stated next to the
 * code that uses them in dynlp_oracle.cpp.
 */
#ifndef DLP_ORACLE_H
#define DLP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_SEMANTICS_REF = 0, ORC_SEMANTICS_SPEC = 1 };

typedef struct orc_batch_in {
  const int *inserted;
  int num_inserted;
  const int *gt_ids;
  const float *gt_labels;
  int num_gt;
  const int *deleted;
  int num_deleted;
  const int *edge_src;
  const int *edge_dst;
  const float *edge_weight;
  int num_edges;
} orc_batch_in;

/* Per-batch results. Field meaning is the same as in the product's
 * dlp_batch_stats (include/dlp_gb300.h). */
typedef struct orc_stats {
  int batch;
  int iterations;        /* propagation passes run (iterationsUsed) */
  int num_components;    /* components among inserted vertices (-1 sentinel excluded) */
  int num_sub_edges;     /* 2 x |new-new edges with w > tau| */
  int hook_edges;        /* edges the connected-components step hooked */
  int hook_truncated;    /* 1 when num_sub_edges exceeded the raw edge count */
  int seed_frontier;     /* |F_0| */
  int seed_marks;        /* vertices marked affected before filtering */
  int64_t affected_edges;  /* sum over passes of the frontier's row lengths */
  int64_t frontier_visits; /* sum over passes of the frontier size */
  int64_t correct;
  int64_t total;
  float accuracy;
  int init_branch;       /* 0 none, 1 component init, 2 no-edge init */
} orc_stats;

/* Artefacts of the last applied batch (for element-wise parity). */
enum {
  ORC_ART_SEED_MARKS = 0,   /* int32 ascending: vertices marked affected (raw) */
  ORC_ART_FRONTIER0 = 1,    /* int32 ascending: F_0 */
  ORC_ART_SUB_EDGES = 2,    /* int32 pairs (u,v),(v,u) in raw edge order */
  ORC_ART_COMP_ROOT = 3,    /* int32 per inserted vertex: min vertex id of its component, -1 sentinel */
  ORC_ART_COMP_ID = 4,      /* int32 per inserted vertex: the reference's sequential component id */
  ORC_ART_INIT_LABELS = 5,  /* fp32 per inserted vertex after initialisation */
  ORC_ART_FRONTIER_SIZES = 6, /* int32 per pass: |F_k| */
  ORC_ART_ROW_PTR = 7,      /* int32 n+1: active CSR of this batch (before soft delete) */
  ORC_ART_COL_IND = 8,      /* int32: active CSR columns (before soft delete) */
  ORC_ART_VALUES = 9,       /* fp32: active CSR weights */
  ORC_ART_LABELS = 10,      /* fp32 n: labels after the batch */
  ORC_ART_STATUS = 11,      /* int32 n: host vertex status after the batch's update */
  ORC_ART_COUNT = 12
};

typedef struct orc_run orc_run;

/* Copies the full graph. batch_map may be NULL (vertex active iff its status is
 * not DELETED); with a map, a vertex is active in batch b only when
 * 0 <= batch_map[v] <= b as well (src/dynLP.cu:143-145,157). tau < 0 selects
 * the mean full-graph edge weight. threads <= 0 means all OpenMP threads. */
orc_run *orc_create(int n, const int *row_ptr, const int *col_ind,
                    const float *values, const float *true_labels,
                    const int *batch_map, float tau, float delta,
                    int max_iterations, int semantics, int threads, int record);
void orc_destroy(orc_run *r);
float orc_tau(const orc_run *r);
/* FP64 modes (set before the first batch).
 * mode 1: the same schedule with every label and every propagation /
 *   initialisation product, sum and quotient in double; orc_labels returns
 *   the double labels rounded to float, orc_labels64 the double labels.
 * mode 2 (shadow): the fp32 run as usual, plus each batch's propagation
 *   repeated in double from the same state (labels after initialisation, the
 *   same first frontier); orc_labels64 returns the shadow's labels after the
 *   batch and orc_shadow_iterations its pass count. This isolates one batch's
 *   fp32 error from the drift of earlier batches.
 * orc_labels64 is NULL in mode 0. */
int orc_set_fp64(orc_run *r, int mode);
const double *orc_labels64(const orc_run *r);
int orc_shadow_iterations(const orc_run *r);
/* Returns 0 on success, nonzero on invalid input (message in orc_error). */
int orc_apply_batch(orc_run *r, int batch_index, const orc_batch_in *in,
                    orc_stats *out);
const char *orc_error(const orc_run *r);
const float *orc_labels(const orc_run *r);
const void *orc_artefact(const orc_run *r, int which, int64_t *count);

/* IrLP full recompute (src/validation.cu:47-208) on a snapshot. status and
 * gt_class are int32 per vertex; labels is updated in place. Returns the number
 * of iterations; edge_visits receives the number of row entries read. */
int orc_irlp(int n, const int *row_ptr, const int *col_ind, const float *values,
             const int *status, const int *gt_class, float *labels, float delta,
             int max_iterations, int threads, int64_t *edge_visits);

/* The reference's input generator, restated (generate_oracle.cpp): full
 * graph, true labels and batches for the given arguments. The batch views
 * point into the problem and stay valid until orc_problem_free. */
typedef struct orc_problem orc_problem;
orc_problem *orc_generate(int n, int avg_degree, int num_batches, unsigned seed,
                          float gt_fraction, float deleted_fraction);
void orc_problem_free(orc_problem *p);
int orc_problem_num_nodes(const orc_problem *p);
int64_t orc_problem_num_edges(const orc_problem *p);
const int *orc_problem_row_ptr(const orc_problem *p);
const int *orc_problem_col_ind(const orc_problem *p);
const float *orc_problem_values(const orc_problem *p);
const float *orc_problem_true_labels(const orc_problem *p);
int orc_problem_num_batches(const orc_problem *p);
int orc_problem_batch(const orc_problem *p, int b, orc_batch_in *out);

#ifdef __cplusplus
}
#endif
#endif
