// Autotuner of the batch engine's launch shape (C ABI dlp_autotune in
// dlp_gb300.h). No counterpart in the reference, whose launch shapes are
// fixed (256-thread blocks, one block per row, src/iterativePropagation.cu).
//
// The engine's propagation splits rows into two degree buckets: rows of at
// most 32 live entries go to groups of `narrow_lanes` lanes (4, 8, 16 or 32;
// or 1: a lane per row of at most 8 entries), longer rows to whole warps. Each pass also picks its launch mode by the
// total frontier: one block (up to solo_entry vertices), a 16-block sub-grid
// (up to subgrid_entry) or the whole grid. The tunables are the lane width of
// the short-row bucket, the two frontier thresholds and the persistent grid's
// blocks per SM (one for the 1,024-thread build): the best choice depends on
// the row lengths and frontier sizes of the workload. The tuner builds a
// sample workload with the reference generator (graph sizes and degrees given
// by the caller), times every candidate on it with CUDA events (the engine's
// own step events), checks that every candidate produced the same statistics
// (the arithmetic does not depend on the launch shape) and keeps the fastest.
#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "session_kernel.cuh"

namespace {

constexpr int kTuneMaxCandidates = 32;  // the report's capacity

struct ProblemDeleter {
  void operator()(dlp_problem *p) const { dlp_problem_free(p); }
};
using ProblemPtr = std::unique_ptr<dlp_problem, ProblemDeleter>;

struct EngineDeleter {
  void operator()(dlp_engine *e) const { dlp_engine_destroy(e); }
};
using EnginePtr = std::unique_ptr<dlp_engine, EngineDeleter>;

// Runs the sample on one candidate; returns device ms and the statistics.
int trial(const dlp_config &cfg, const std::vector<ProblemPtr> &probs, int batches,
          const std::vector<std::vector<int>> &bmaps, double *ms, std::vector<dlp_batch_stats> *stats) {
  dlp_engine *raw = nullptr;
  DLP_TRY(dlp_engine_create(&cfg, static_cast<int>(probs.size()), 0, &raw));
  EnginePtr eng(raw);
  std::vector<int> gids(probs.size());
  for (size_t i = 0; i < probs.size(); ++i) {
    dlp_problem *p = probs[i].get();
    DLP_TRY(dlp_engine_add_graph(raw, dlp_problem_num_nodes(p), dlp_problem_num_edges(p), dlp_problem_row_ptr(p),
                                 dlp_problem_col_ind(p), dlp_problem_values(p), dlp_problem_true_labels(p),
                                 bmaps[i].data(), &gids[i]));
  }
  const int first = dlp_engine_steps(raw);
  stats->clear();
  for (int b = 0; b < batches; ++b) {
    std::vector<int> g, bi;
    std::vector<dlp_batch_view> v;
    for (size_t i = 0; i < probs.size(); ++i) {
      if (b >= dlp_problem_num_batches(probs[i].get())) continue;
      dlp_batch_view bv;
      DLP_TRY(dlp_problem_batch(probs[i].get(), b, &bv));
      g.push_back(gids[i]);
      bi.push_back(b);
      v.push_back(bv);
    }
    if (g.empty()) continue;
    std::vector<dlp_batch_stats> st(g.size());
    DLP_TRY(dlp_engine_step(raw, static_cast<int>(g.size()), g.data(), bi.data(), v.data(), st.data()));
    stats->insert(stats->end(), st.begin(), st.end());
  }
  // sum of the steps' own device times (the host's staging between steps is
  // not part of a candidate's cost)
  double total = 0.0;
  for (int s = first; s < dlp_engine_steps(raw); ++s) {
    float t = 0.0f;
    DLP_TRY(dlp_engine_elapsed_ms(raw, s, s, &t));
    total += t;
  }
  *ms = total;
  return DLP_OK;
}

bool same_stats(const std::vector<dlp_batch_stats> &a, const std::vector<dlp_batch_stats> &b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); ++i) {
    const dlp_batch_stats &x = a[i], &y = b[i];
    if (x.iterations != y.iterations || x.num_components != y.num_components || x.affected_edges != y.affected_edges ||
        x.frontier_visits != y.frontier_visits || x.correct != y.correct || x.total != y.total)
      return false;
  }
  return true;
}

}  // namespace

extern "C" {

int dlp_autotune(dlp_config *cfg, int num_graphs, const int *sizes, const int *degrees, int batches,
                 int max_iterations, dlp_tune_report *report) {
  dlp::clear_error();
  if (!cfg || num_graphs <= 0 || num_graphs > 1024 || !sizes || !degrees || batches <= 0 || max_iterations <= 0)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "invalid autotune arguments");
  std::vector<ProblemPtr> probs;
  std::vector<std::vector<int>> bmaps;
  for (int i = 0; i < num_graphs; ++i) {
    dlp_problem *p = nullptr;
    DLP_TRY(dlp_problem_generate(sizes[i], degrees[i], batches, 1000u + static_cast<unsigned>(i), 0.01f, 0.09f, &p));
    probs.emplace_back(p);
    // arrival batch per vertex, as the reference's host rebuild uses it
    std::vector<int> m(dlp_problem_num_nodes(p), -1);
    for (int b = 0; b < dlp_problem_num_batches(p); ++b) {
      dlp_batch_view v;
      DLP_TRY(dlp_problem_batch(p, b, &v));
      for (int k = 0; k < v.num_inserted; ++k) m[v.inserted[k]] = b;
    }
    bmaps.push_back(std::move(m));
  }
  static const int kLanes[] = {1, 4, 8};
  static const int kSoloEntries[] = {256, 512, 1024};
  static const int kSubEntries[] = {1024, 2048, 4096};
  // blocks per SM the build's block size allows (1024-thread blocks: one)
  std::vector<int> kBlocks = {1};
  if (dlp::session::kBlock <= 512) kBlocks.insert(kBlocks.begin(), 2);
  dlp_tune_report rep;
  std::memset(&rep, 0, sizeof(rep));
  std::vector<dlp_batch_stats> ref_stats;
  double best = -1.0;
  for (int bl : kBlocks)
    for (int ln : kLanes)
      for (int se : kSoloEntries)
        for (int ge : kSubEntries) {
          if (rep.candidates >= kTuneMaxCandidates) break;
          dlp_config c = *cfg;
          c.narrow_lanes = ln;
          c.blocks_per_sm = bl;
          c.solo_entry = se;
          c.subgrid_entry = ge;
          c.max_iterations = max_iterations;
          c.record = 0;
          double ms = 0.0;
          std::vector<dlp_batch_stats> st;
          DLP_TRY(trial(c, probs, batches, bmaps, &ms, &st));
          if (ref_stats.empty()) ref_stats = st;
          else if (!same_stats(ref_stats, st))
            return dlp::fail(DLP_ERR_INTERNAL, "launch shapes disagree on the sample's statistics");
          const int k = rep.candidates++;
          rep.lanes[k] = ln;
          rep.blocks_per_sm[k] = bl;
          rep.solo_entry[k] = se;
          rep.subgrid_entry[k] = ge;
          rep.ms[k] = ms;
          if (best < 0.0 || ms < best) {
            best = ms;
            rep.best = k;
          }
        }
  cfg->narrow_lanes = rep.lanes[rep.best];
  cfg->blocks_per_sm = rep.blocks_per_sm[rep.best];
  cfg->solo_entry = rep.solo_entry[rep.best];
  cfg->subgrid_entry = rep.subgrid_entry[rep.best];
  if (report) *report = rep;
  return DLP_OK;
}

}  // extern "C"
