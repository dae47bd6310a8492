// Test infrastructure, not product code: the oracle's own restatement of the
// reference's input generator, so that CPU-side checks and the CPU baseline can
// build their inputs without loading the product library.
//
// It makes the same libstdc++ <random> calls in the same order as the
// reference, with the same containers where order matters:
//   graph    src/generateSparseGraph.cu:118-215 (balanced labels shuffled, a
//            spanning tree over a shuffled permutation, uniform extra edges
//            deduplicated in a std::set, class-dependent weights; then
//            :51-110, CSR filled in edge-list order and each row
//            insertion-sorted by column)
//   batches  src/generateBatches.cu:44-207 (balanced ground truth in batch 0,
//            the rest shuffled and split evenly, a ground-truth share of each
//            batch, every edge in the batch of its later endpoint, deletions
//            drawn from the active non-ground-truth set in ascending order)
// Fractions are multiplied in float, as the reference does with its float
// config fields. tests/test_golden_inputs.py checks the output against the
// reference's own generator.
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <random>
#include <set>
#include <utility>
#include <vector>

#include "oracle.h"

struct orc_problem {
  int n = 0;
  std::vector<int> row_ptr, col;
  std::vector<float> val, truth;
  struct B {
    std::vector<int> ins, gt_ids, del, es, ed;
    std::vector<float> gt_lab, ew;
  };
  std::vector<B> batches;
};

namespace {

float class_weight(std::mt19937 &rng, bool same) {
  std::uniform_real_distribution<float> same_d(0.5f, 1.0f), cross_d(0.01f, 0.5f);
  return same ? same_d(rng) : cross_d(rng);
}

void make_graph(orc_problem &p, int n, int deg, unsigned seed) {
  std::mt19937 rng(seed);
  p.n = n;
  p.truth.resize(n);
  for (int i = 0; i < n; ++i) p.truth[i] = i < n / 2 ? 0.0f : 1.0f;
  std::shuffle(p.truth.begin(), p.truth.end(), rng);
  std::vector<int> perm(n);
  std::iota(perm.begin(), perm.end(), 0);
  std::shuffle(perm.begin(), perm.end(), rng);

  std::set<std::pair<int, int>> seen;
  std::vector<std::pair<int, int>> edges;
  std::vector<float> w;
  for (int i = 0; i + 1 < n; ++i) {
    const int a = std::min(perm[i], perm[i + 1]), b = std::max(perm[i], perm[i + 1]);
    seen.insert({a, b});
    edges.push_back({a, b});
    w.push_back(class_weight(rng, p.truth[a] == p.truth[b]));
  }
  long long target = static_cast<long long>(n) * deg / 2;
  if (target < n - 1) target = n - 1;
  std::uniform_int_distribution<int> pick(0, n - 1);
  const int max_attempts = static_cast<int>(target) * 10;
  int attempts = 0;
  while (static_cast<long long>(edges.size()) < target && attempts < max_attempts) {
    const int u = pick(rng), v = pick(rng);
    if (u == v) {
      ++attempts;
      continue;
    }
    const int a = std::min(u, v), b = std::max(u, v);
    if (!seen.insert({a, b}).second) {
      ++attempts;
      continue;
    }
    edges.push_back({a, b});
    w.push_back(class_weight(rng, p.truth[a] == p.truth[b]));
    attempts = 0;
  }

  std::vector<int> deg_of(n, 0);
  for (const auto &e : edges) {
    ++deg_of[e.first];
    ++deg_of[e.second];
  }
  p.row_ptr.assign(static_cast<size_t>(n) + 1, 0);
  for (int i = 0; i < n; ++i) p.row_ptr[i + 1] = p.row_ptr[i] + deg_of[i];
  p.col.resize(p.row_ptr[n]);
  p.val.resize(p.row_ptr[n]);
  std::vector<int> fill(p.row_ptr.begin(), p.row_ptr.end() - 1);
  for (size_t k = 0; k < edges.size(); ++k) {
    const int a = edges[k].first, b = edges[k].second;
    p.col[fill[a]] = b;
    p.val[fill[a]++] = w[k];
    p.col[fill[b]] = a;
    p.val[fill[b]++] = w[k];
  }
  // stable per-row sort by column (an insertion sort keeps equal keys in
  // order; columns in a row are distinct anyway)
  for (int u = 0; u < n; ++u) {
    const int s = p.row_ptr[u], e = p.row_ptr[u + 1];
    std::vector<std::pair<int, float>> row;
    for (int k = s; k < e; ++k) row.push_back({p.col[k], p.val[k]});
    std::stable_sort(row.begin(), row.end(), [](const auto &x, const auto &y) { return x.first < y.first; });
    for (int k = s; k < e; ++k) {
      p.col[k] = row[k - s].first;
      p.val[k] = row[k - s].second;
    }
  }
}

void make_batches(orc_problem &p, int nb, unsigned seed, float gt_frac, float del_frac) {
  const int n = p.n;
  std::mt19937 rng(seed + 12345u);
  std::vector<int> c0, c1;
  for (int i = 0; i < n; ++i) (p.truth[i] < 0.5f ? c0 : c1).push_back(i);
  std::shuffle(c0.begin(), c0.end(), rng);
  std::shuffle(c1.begin(), c1.end(), rng);
  p.batches.assign(nb, {});
  const int initial = std::max(2, static_cast<int>(static_cast<float>(n) * gt_frac));
  const int per_class = initial / 2;
  std::vector<char> is_gt0(n, 0);
  auto &b0 = p.batches[0];
  for (int c = 0; c < 2; ++c) {
    const std::vector<int> &cls = c == 0 ? c0 : c1;
    for (int i = 0; i < per_class && i < static_cast<int>(cls.size()); ++i) {
      b0.ins.push_back(cls[i]);
      b0.gt_ids.push_back(cls[i]);
      b0.gt_lab.push_back(c == 0 ? 0.0f : 1.0f);
      is_gt0[cls[i]] = 1;
    }
  }
  std::vector<int> rest;
  for (int i = 0; i < n; ++i)
    if (!is_gt0[i]) rest.push_back(i);
  std::shuffle(rest.begin(), rest.end(), rng);
  const int groups = std::max(1, nb - 1);
  const int per = static_cast<int>(rest.size()) / groups;
  const int extra = static_cast<int>(rest.size()) - per * groups;
  size_t at = 0;
  for (int b = 1; b < nb; ++b) {
    auto &bt = p.batches[b];
    const int cnt = per + (b <= extra ? 1 : 0);
    for (int j = 0; j < cnt && at < rest.size(); ++j) bt.ins.push_back(rest[at++]);
    const int ngt = std::max(1, static_cast<int>(static_cast<float>(bt.ins.size()) * gt_frac));
    std::vector<int> mix = bt.ins;
    std::shuffle(mix.begin(), mix.end(), rng);
    for (int j = 0; j < ngt && j < static_cast<int>(mix.size()); ++j) {
      bt.gt_ids.push_back(mix[j]);
      bt.gt_lab.push_back(p.truth[mix[j]]);
    }
  }
  std::vector<int> arrive(n, -1);
  for (int b = 0; b < nb; ++b)
    for (int v : p.batches[b].ins) arrive[v] = b;
  for (int u = 0; u < n; ++u) {
    if (arrive[u] < 0) continue;
    for (int k = p.row_ptr[u]; k < p.row_ptr[u + 1]; ++k) {
      const int v = p.col[k];
      if (v < 0 || arrive[v] < 0 || u >= v) continue;
      auto &bt = p.batches[std::max(arrive[u], arrive[v])];
      bt.es.push_back(u);
      bt.ed.push_back(v);
      bt.ew.push_back(p.val[k]);
    }
  }
  std::set<int> gt_all(p.batches[0].gt_ids.begin(), p.batches[0].gt_ids.end());
  std::set<int> active;
  for (int b = 1; b < nb; ++b) {
    auto &bt = p.batches[b];
    gt_all.insert(bt.gt_ids.begin(), bt.gt_ids.end());
    for (int v : bt.ins)
      if (!gt_all.count(v)) active.insert(v);
    int ndel = static_cast<int>(static_cast<float>(bt.ins.size()) * del_frac);
    ndel = std::min(ndel, static_cast<int>(active.size()));
    if (ndel > 0) {
      std::vector<int> cand(active.begin(), active.end());
      std::shuffle(cand.begin(), cand.end(), rng);
      for (int j = 0; j < ndel; ++j) {
        bt.del.push_back(cand[j]);
        active.erase(cand[j]);
      }
    }
  }
}

}  // namespace

extern "C" {

orc_problem *orc_generate(int n, int avg_degree, int num_batches, unsigned seed, float gt_fraction,
                          float deleted_fraction) {
  if (n <= 1 || avg_degree <= 0 || num_batches <= 0) return nullptr;
  orc_problem *p = new orc_problem();
  make_graph(*p, n, avg_degree, seed);
  make_batches(*p, num_batches, seed, gt_fraction, deleted_fraction);
  return p;
}

void orc_problem_free(orc_problem *p) { delete p; }
int orc_problem_num_nodes(const orc_problem *p) { return p->n; }
int64_t orc_problem_num_edges(const orc_problem *p) { return static_cast<int64_t>(p->col.size()); }
const int *orc_problem_row_ptr(const orc_problem *p) { return p->row_ptr.data(); }
const int *orc_problem_col_ind(const orc_problem *p) { return p->col.data(); }
const float *orc_problem_values(const orc_problem *p) { return p->val.data(); }
const float *orc_problem_true_labels(const orc_problem *p) { return p->truth.data(); }
int orc_problem_num_batches(const orc_problem *p) { return static_cast<int>(p->batches.size()); }

int orc_problem_batch(const orc_problem *p, int b, orc_batch_in *out) {
  if (b < 0 || b >= static_cast<int>(p->batches.size()) || !out) return 1;
  const auto &bt = p->batches[b];
  out->inserted = bt.ins.data();
  out->num_inserted = static_cast<int>(bt.ins.size());
  out->gt_ids = bt.gt_ids.data();
  out->gt_labels = bt.gt_lab.data();
  out->num_gt = static_cast<int>(bt.gt_ids.size());
  out->deleted = bt.del.data();
  out->num_deleted = static_cast<int>(bt.del.size());
  out->edge_src = bt.es.data();
  out->edge_dst = bt.ed.data();
  out->edge_weight = bt.ew.data();
  out->num_edges = static_cast<int>(bt.es.size());
  return 0;
}

}  // extern "C"
