// Multi-graph batch engine: one cooperative persistent kernel applies one
// batch to each of up to kMaxGraphs resident graphs at once.
//
// Every phase of the per-batch update (see session_kernel.cuh for the phase
// map against the reference) walks a flattened work list: the per-graph item
// counts are prefix-summed in shared memory after each grid barrier and a
// work item is mapped back to (graph, local index) by binary search. Graphs
// converge independently: a graph whose frontier is empty (or that reached
// max_iter) contributes no items to later passes and its pass count is
// recorded; the launch ends when every graph has finished. A resident single
// graph (dlp_session) is the one-graph case of the same kernel.
#pragma once

#include "session_kernel.cuh"

namespace dlp {
namespace engine {

constexpr int kMaxGraphs = 1024;

struct GraphRec {
  session::DevState st;
  session::BatchArgs ba;
};

struct EngineCtl {
  GridBarrier bar;      // all blocks of the launch
  GridBarrier sub_bar;  // the first blocks only (sub-grid passes)
  int err;
  int solo_k;           // pass at which the last solo / sub-grid stint handed back
  int solo_passes;      // passes that stint ran
  int sub_stop;         // first pass + 1 of a sub-grid stint that ran out of time
  int where;            // last phase block 0 reached (1..10)
  int where_pass;       // last propagation pass block 0 started
};

struct EngineArgs {
  GraphRec *recs;
  int ng;
  EngineCtl *ectl;
  unsigned long long timeout_ns;
  int solo;  // bit 0: one-block passes for small frontiers; bit 1: sub-grid passes
};

const void *engine_kernel_ptr(int lanes);
// Dynamic shared memory per block of the engine kernel (the solo-mode cache).
size_t engine_dynamic_smem();

}  // namespace engine
}  // namespace dlp
