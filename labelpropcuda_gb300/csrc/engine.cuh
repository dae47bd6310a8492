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
//
// Continuous batching: a launch may be sliced (a pass budget or a time budget
// for its propagation). Graphs whose frontier is still live when the slice
// ends keep their whole propagation state in device memory (frontier sets,
// counters, both label buffers) and are continued by a later launch, which
// lists them after the graphs that start a new batch: phases A-F run over the
// new graphs only, the propagation passes over all of them, each graph at its
// own pass number (BatchArgs::pass0 + the launch's pass). A graph's batch ends
// (phase H, statistics) in the launch where its frontier empties.
#pragma once

#include "session_kernel.cuh"

namespace dlp {
namespace engine {

constexpr int kMaxGraphs = 1024;
// Frontier sizes below which propagation passes leave the full grid: the
// one-block mode (default 512, at most kSoloEntryMax) and the 16-block
// sub-grid mode (default 2048, at most kSubEntryMax). Tunable per engine.
constexpr int kSoloEntryDefault = 512;
constexpr int kSoloEntryMax = 1024;
constexpr int kSubEntryDefault = 2048;
constexpr int kSubEntryMax = 4096;
constexpr int kSubLive = 4096;  // the sub-grid mode leaves once the frontier grows above this

struct GraphRec {
  session::DevState st;
  session::BatchArgs ba;
};

struct EngineCtl {
  GridBarrier bar;      // all blocks of the launch
  GridBarrier sub_bar;  // the first blocks only (sub-grid passes)
  int err;
  // Hand-back of a solo / sub-grid stint: the pass at which it stopped and the
  // passes it ran, in slot (stint number & 1), so that the next stint cannot
  // overwrite a value a slow block has yet to read.
  int solo_k[2];
  int solo_passes[2];
  // Stop requests, written by thread 0 of block 0 and read by every block at
  // the top of a pass: (launch tag << 32) | the pass at which to stop. A read
  // at the top of pass k takes only a request naming pass k, so a request
  // written during pass k (for pass k + 1) is never seen early by a block that
  // is slow to start pass k.
  unsigned long long sub_stop;    // a sub-grid stint ran out of time
  int where;            // last phase block 0 reached (1..10)
  int where_pass;       // last propagation pass block 0 started
  unsigned long long slice_stop;  // the launch's time slice ran out
  unsigned long long t_launch;  // global timer at the start of the launch (thread 0 of block 0)
  // Propagation passes run so far by mode, and the device time they took
  // (global timer): 0 one block, 1 of which the 8-warp team, 2 sub-grid,
  // 3 full grid. Written by thread 0 of block 0 only, once per launch.
  unsigned long long mode_passes[4];
  unsigned long long mode_ns[4];
};

struct EngineArgs {
  GraphRec *recs;
  int ng;       // graphs in the launch
  int ng_new;   // the first ng_new of them start a batch; the rest continue one
  EngineCtl *ectl;
  unsigned long long timeout_ns;
  int solo;  // bit 0: one-block passes; bit 1: sub-grid passes; bit 2: team passes
  int fast_div;    // 1: the reference's fast-math division (dlp_config.arithmetic), else IEEE
  int solo_entry;  // total frontier at most this: one-block passes (<= kSoloEntryMax)
  int sub_entry;   // total frontier at most this: sub-grid passes (<= kSubLive)
  int pass_budget;                // propagation passes this launch runs at most (0: no limit)
  unsigned long long slice_ns;    // propagation time after which the launch stops (0: no limit)
  int tag;                        // unique per launch (stop requests)
  float delta;                    // convergence threshold (the engine's, the same for every graph)
  int2 *progress;                 // per graph: {1 batch finished / 0 continues, passes so far}
};

// Zeroes the batch counters of the graphs that start a batch (recs[0..ng_new)).
void launch_zero_counters(const GraphRec *recs, int ng_new, cudaStream_t stream);

const void *engine_kernel_ptr(int lanes);
// Dynamic shared memory per block of the engine kernel (the solo-mode cache).
size_t engine_dynamic_smem();

}  // namespace engine
}  // namespace dlp
