// Per-graph device state and per-batch arguments of the batch engine
// (engine.cuh, engine_kernel.cu). The whole per-batch update of a dynamic
// graph runs inside ONE cooperative persistent launch, shared with the other
// graphs of the step; phases are separated by grid barriers and nothing
// returns to the host inside a batch.
//
// Reference path replaced (SMShovan/LabelPropCUDA, src/dynLP.cu:284-558):
//   host rebuild + re-upload of the active CSR  -> phases A-C (incremental,
//                                                  only rows next to changed vertices)
//   markDeletions / cleanIncomingEdges          -> phase C (soft delete in place)
//   count/build sparsified subgraph             -> phase C (tau filter, marks)
//   Shiloach-Vishkin components                 -> phase D (atomicMin hook +
//                                                  pointer-jumping compress)
//   supernode weights + label init              -> phases E-F
//   collect / propagate / markNeighbors loop    -> phase G (frontier lists
//                                                  rebuilt by stamp atomics)
//   enforce ground truth + host accuracy        -> phase H (incremental counters)
#pragma once

#include "common.cuh"

namespace dlp {
namespace session {

#ifndef DLP_BLOCK
#define DLP_BLOCK 1024
#endif
constexpr int kBlock = DLP_BLOCK;       // threads per block of the persistent kernel (512 or 1024)
static_assert(kBlock == 512 || kBlock == 1024, "the persistent kernel is tuned for 512 or 1024 threads");
constexpr int kMaxHookRounds = 100;     // the reference's outer SV cap (src/connectedComponents.cu:209)
constexpr int kRecordIters = 1 << 17;   // per-pass frontier sizes kept when recording
constexpr int kNarrowMax = 32;          // rows up to this length use the group path
constexpr int kRowGroup = 8;            // lanes per row in the bookkeeping phases

// Per-batch counters of one graph, zeroed at the start of the launch that
// begins the graph's batch (they carry over when its propagation is continued
// by later launches).
struct BatchCounters {
  int front_count[3][2];  // frontier list sets: [set][0 narrow, 1 wide]
  int num_dirty;
  int num_seeds;
  int num_kept;           // new-new edges with w > tau
  int num_comp;
  int seed_frontier;
  int hook_rounds;
  int passes;             // propagation passes this graph ran
  int hook_flag[kMaxHookRounds];
  unsigned long long aff_edges;
  unsigned long long front_visits;
  unsigned long long dirty_entries;
};

// Session state that persists across batches.
struct SessionCtl {
  GridBarrier bar;
  int err;                  // sticky device error (DLP_ERR_*)
  int cur_buf;              // which label buffer holds the current labels
  unsigned stamp_base;      // frontier stamps used so far
  int touched_count[2];     // vertices written by propagation, per batch parity
  long long correct;        // accuracy counters over active non-GT vertices
  long long total;
};

struct DevState {
  int n;
  const int *full_row;      // n+1, full graph
  const int2 *full_adj;     // {col, weight bits}, full graph
  int2 *act_adj;            // live rows, same slots as full_adj
  int *act_len;             // live row length
  int2 *rowinfo;            // {row start, live row length}: what a propagation pass reads, in one load
  int8_t *status;           // host-side status (src/dynLP.cu:117-130)
  int8_t *gt;               // -1 / 0 / 1
  uint8_t *nmeta;           // what propagation needs about a neighbour, in one byte:
                            // bit 0 markable (no ground truth), bit 1 live row longer than 32
  const uint8_t *truth;     // 0 / 1
  int *contrib;             // accuracy contribution: -1 none, 0 wrong, 1 right
  const int *batch_map;     // arrival batch per vertex, or null
  float *lab0, *lab1;
  int *local;               // vertex -> position in this batch's inserted list
  unsigned *del_stamp, *gt_stamp, *dirty_stamp, *front_stamp;
  int *dirty_list;          // n
  int *seed_list;           // n
  int *flist;               // 3n: frontier sets (narrow from the front, wide from the back)
  int *touched;             // 2n
  int *par;                 // n: SV parent over inserted positions
  long long *acc;           // 2n: fixed-point supernode weights per root position
  int *lsrc, *ldst;         // per raw edge: inserted position or -1
  int *sub_pairs;           // kept edges: (src,dst) global ids
  int *sub_local;           // kept edges: (src,dst) inserted positions
  int *del_pre;             // spec: status before the batch, per deleted entry
  int *del_keep;            // this batch's deletions, read by the next batch
  SessionCtl *ctl;
  BatchCounters *bc;
  dlp_batch_stats *stats_slot;
  // recording (null unless requested)
  int *rec_front0;
  int *rec_root;
  float *rec_init;
  int *rec_fsizes;
  int *rec_minid;
};

struct BatchArgs {
  int batch;                // the caller's batch index (vertex_batch_map test)
  int seq;                  // batches applied since reset
  const int *ins;
  int I;
  const int *gt_ids;
  const float *gt_lab;
  int G;
  const int *del;
  int D;
  const int *es;
  const int *ed;
  const float *ew;
  int E;
  const int *prev_del;
  int PD;
  float tau;
  float delta;
  int max_iter;
  int spec;
  int record;
  int solo;                 // small frontiers run on one block (see phase G)
  int pass0;                // propagation passes run by earlier launches (0: batch starts here)
  unsigned long long timeout_ns;
};

}  // namespace session
}  // namespace dlp
