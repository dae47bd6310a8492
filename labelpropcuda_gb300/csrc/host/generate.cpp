// Deterministic synthetic input pipeline: graph, true labels and batches.
//
// The reference draws its inputs with libstdc++ <random> (std::mt19937,
// std::shuffle, uniform_{int,real}_distribution). The draws are reproduced here
// call for call, so a seed gives the same graph and batches as the reference
// binary. What differs is the bookkeeping around the draws: duplicate edges are
// found with an open-addressing hash set instead of std::set<pair<int,int>>,
// the CSR rows are sorted with std::sort (column ids in a row are unique, so
// the order equals the reference's insertion sort), and the deletion
// candidates are kept in a flag array scanned in ascending id order (the order
// in which std::set<int> iterates). The accept/reject decisions, and therefore
// the RNG stream, are unchanged.
//
// Built with -ffp-contract=off: libstdc++'s generate_canonical has a
// multiply-add that must not become an FMA on aarch64.

#include "problem.h"

#include <algorithm>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <numeric>
#include <random>
#include <sstream>
#include <utility>

namespace dlp {
namespace {

// Open-addressing set of undirected edges keyed by (min << 32 | max).
class EdgeSet {
 public:
  explicit EdgeSet(int64_t expected) {
    uint64_t cap = 16;
    while (cap < static_cast<uint64_t>(expected) * 2 + 16) cap <<= 1;
    slots_.assign(cap, kEmpty);
    mask_ = cap - 1;
  }
  // Returns true when the key was absent (and is now present).
  bool insert(uint64_t key) {
    uint64_t i = mix(key) & mask_;
    while (true) {
      uint64_t s = slots_[i];
      if (s == key) return false;
      if (s == kEmpty) {
        slots_[i] = key;
        return true;
      }
      i = (i + 1) & mask_;
    }
  }
  bool contains(uint64_t key) const {
    uint64_t i = mix(key) & mask_;
    while (true) {
      uint64_t s = slots_[i];
      if (s == key) return true;
      if (s == kEmpty) return false;
      i = (i + 1) & mask_;
    }
  }

 private:
  static constexpr uint64_t kEmpty = ~0ull;
  static uint64_t mix(uint64_t x) {  // splitmix64 finaliser
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
  }
  std::vector<uint64_t> slots_;
  uint64_t mask_ = 0;
};

inline uint64_t edge_key(int a, int b) {
  return (static_cast<uint64_t>(static_cast<uint32_t>(a)) << 32) |
         static_cast<uint32_t>(b);
}

// Undirected edge list -> CSR with both directions, each row sorted by column.
void build_csr(int n, const std::vector<std::pair<int, int>> &edges,
               const std::vector<float> &w, HostGraph &g) {
  std::vector<int> deg(n, 0);
  for (const auto &e : edges) {
    ++deg[e.first];
    ++deg[e.second];
  }
  g.n = n;
  g.row_ptr.assign(static_cast<size_t>(n) + 1, 0);
  for (int i = 0; i < n; ++i) g.row_ptr[i + 1] = g.row_ptr[i] + deg[i];
  const size_t m = static_cast<size_t>(g.row_ptr[n]);
  g.col.assign(m, 0);
  g.val.assign(m, 0.0f);
  std::vector<int> fill(g.row_ptr.begin(), g.row_ptr.end() - 1);
  for (size_t i = 0; i < edges.size(); ++i) {
    const int a = edges[i].first, b = edges[i].second;
    g.col[fill[a]] = b;
    g.val[fill[a]++] = w[i];
    g.col[fill[b]] = a;
    g.val[fill[b]++] = w[i];
  }
  std::vector<std::pair<int, float>> row;
#pragma omp parallel for schedule(dynamic, 4096) private(row)
  for (int u = 0; u < n; ++u) {
    const int s = g.row_ptr[u], e = g.row_ptr[u + 1];
    if (e - s < 2) continue;
    row.clear();
    for (int k = s; k < e; ++k) row.emplace_back(g.col[k], g.val[k]);
    std::sort(row.begin(), row.end(),
              [](const std::pair<int, float> &x, const std::pair<int, float> &y) {
                return x.first < y.first;
              });
    for (int k = s; k < e; ++k) {
      g.col[k] = row[k - s].first;
      g.val[k] = row[k - s].second;
    }
  }
}

}  // namespace

bool generate_graph(int n, int avg_degree, unsigned seed, HostGraph &g,
                    std::vector<float> &truth, std::string *err) {
  if (n <= 1) {
    if (err) *err = "totalNodes must be > 1";
    return false;
  }
  if (avg_degree <= 0) {
    if (err) *err = "avgDegree must be positive";
    return false;
  }
  std::mt19937 rng(seed);

  // Balanced classes, shuffled.
  truth.resize(n);
  for (int i = 0; i < n; ++i) truth[i] = (i < n / 2) ? 0.0f : 1.0f;
  std::shuffle(truth.begin(), truth.end(), rng);

  std::vector<int> perm(n);
  std::iota(perm.begin(), perm.end(), 0);
  std::shuffle(perm.begin(), perm.end(), rng);

  int64_t target = static_cast<int64_t>(n) * avg_degree / 2;
  if (target < static_cast<int64_t>(n) - 1) target = n - 1;

  std::uniform_real_distribution<float> same_class(0.5f, 1.0f);
  std::uniform_real_distribution<float> cross_class(0.01f, 0.5f);
  auto draw_weight = [&](int a, int b) {
    return truth[a] == truth[b] ? same_class(rng) : cross_class(rng);
  };

  EdgeSet seen(target);
  std::vector<std::pair<int, int>> edges;
  std::vector<float> w;
  edges.reserve(static_cast<size_t>(target));
  w.reserve(static_cast<size_t>(target));

  // Path over the permutation: a spanning tree.
  for (int i = 0; i + 1 < n; ++i) {
    const int a = std::min(perm[i], perm[i + 1]);
    const int b = std::max(perm[i], perm[i + 1]);
    if (a == b) continue;
    seen.insert(edge_key(a, b));
    w.push_back(draw_weight(a, b));
    edges.emplace_back(a, b);
  }

  // Uniform extra edges; rejected draws (self loops, duplicates) count towards
  // a give-up limit that resets on every accepted edge.
  std::uniform_int_distribution<int> pick(0, n - 1);
  int attempts = 0;
  const int max_attempts = static_cast<int>(target) * 10;
  while (static_cast<int64_t>(edges.size()) < target && attempts < max_attempts) {
    const int x = pick(rng);
    const int y = pick(rng);
    if (x == y) {
      ++attempts;
      continue;
    }
    const int a = std::min(x, y), b = std::max(x, y);
    if (!seen.insert(edge_key(a, b))) {
      ++attempts;
      continue;
    }
    w.push_back(draw_weight(a, b));
    edges.emplace_back(a, b);
    attempts = 0;
  }

  build_csr(n, edges, w, g);
  return true;
}

bool generate_batches(const HostGraph &g, const std::vector<float> &truth,
                      int num_batches, unsigned seed, float gt_fraction,
                      float deleted_fraction, std::vector<HostBatch> &out,
                      std::string *err) {
  const int n = g.n;
  if (num_batches <= 0 || n <= 0) {
    if (err) *err = "invalid numBatches or totalNodes";
    return false;
  }
  std::mt19937 rng(seed + 12345u);

  std::vector<int> class0, class1;
  for (int i = 0; i < n; ++i) (truth[i] < 0.5f ? class0 : class1).push_back(i);
  std::shuffle(class0.begin(), class0.end(), rng);
  std::shuffle(class1.begin(), class1.end(), rng);

  // Batch 0: the initial ground truth, half from each class. The products are
  // float products, as in the reference (int * float).
  const int initial_gt = std::max(2, static_cast<int>(static_cast<float>(n) * gt_fraction));
  const int per_class = initial_gt / 2;
  out.assign(num_batches, HostBatch{});
  std::vector<uint8_t> is_gt(n, 0);
  for (int c = 0; c < 2; ++c) {
    const std::vector<int> &pool = c == 0 ? class0 : class1;
    for (int i = 0; i < per_class && i < static_cast<int>(pool.size()); ++i) {
      const int v = pool[i];
      out[0].inserted.push_back(v);
      out[0].gt_ids.push_back(v);
      out[0].gt_labels.push_back(c == 0 ? 0.0f : 1.0f);
      is_gt[v] = 1;
    }
  }

  // Everything else, shuffled and dealt evenly over batches 1..B-1.
  std::vector<int> rest;
  rest.reserve(n);
  for (int i = 0; i < n; ++i)
    if (!is_gt[i]) rest.push_back(i);
  std::shuffle(rest.begin(), rest.end(), rng);
  const int rest_n = static_cast<int>(rest.size());
  const int slots = std::max(1, num_batches - 1);
  const int per_batch = rest_n / slots;
  const int leftover = rest_n - per_batch * slots;
  int next = 0;
  std::vector<int> pick;
  for (int b = 1; b < num_batches; ++b) {
    const int count = per_batch + (b <= leftover ? 1 : 0);
    for (int j = 0; j < count && next < rest_n; ++j) out[b].inserted.push_back(rest[next++]);
    const int batch_gt = std::max(
        1, static_cast<int>(static_cast<float>(out[b].inserted.size()) * gt_fraction));
    pick = out[b].inserted;
    std::shuffle(pick.begin(), pick.end(), rng);
    for (int j = 0; j < batch_gt && j < static_cast<int>(pick.size()); ++j) {
      out[b].gt_ids.push_back(pick[j]);
      out[b].gt_labels.push_back(truth[pick[j]]);
    }
  }

  // Each edge belongs to the batch of its later endpoint; rows are walked in
  // ascending vertex order and each undirected edge is taken once (u < v).
  std::vector<int> arrival(n, -1);
  for (int b = 0; b < num_batches; ++b)
    for (int v : out[b].inserted) arrival[v] = b;
  for (int u = 0; u < n; ++u) {
    if (arrival[u] < 0) continue;
    for (int k = g.row_ptr[u]; k < g.row_ptr[u + 1]; ++k) {
      const int v = g.col[k];
      if (v < 0 || arrival[v] < 0 || u >= v) continue;
      HostBatch &hb = out[std::max(arrival[u], arrival[v])];
      hb.edge_src.push_back(u);
      hb.edge_dst.push_back(v);
      hb.edge_w.push_back(g.val[k]);
    }
  }

  // Deletions for batches 1..B-1: drawn from the live non-GT vertices,
  // candidates listed in ascending id order before the shuffle.
  std::vector<uint8_t> live(n, 0);
  int64_t live_count = 0;
  std::vector<int> candidates;
  for (int b = 1; b < num_batches; ++b) {
    for (int v : out[b].gt_ids) is_gt[v] = 1;
    for (int v : out[b].inserted)
      if (!is_gt[v] && !live[v]) {
        live[v] = 1;
        ++live_count;
      }
    int to_delete = static_cast<int>(static_cast<float>(out[b].inserted.size()) * deleted_fraction);
    if (static_cast<int64_t>(to_delete) > live_count) to_delete = static_cast<int>(live_count);
    if (to_delete > 0) {
      candidates.clear();
      for (int v = 0; v < n; ++v)
        if (live[v]) candidates.push_back(v);
      std::shuffle(candidates.begin(), candidates.end(), rng);
      for (int j = 0; j < to_delete; ++j) {
        const int v = candidates[j];
        out[b].deleted.push_back(v);
        live[v] = 0;
        --live_count;
      }
    }
  }
  return true;
}

bool write_csr_files(const HostGraph &g, const std::vector<float> &truth,
                     const std::string &prefix, std::string *err) {
  auto open = [&](const char *what, std::ofstream &f) {
    f.open(prefix + what);
    if (!f.is_open()) {
      if (err) *err = std::string("could not write ") + prefix + what;
      return false;
    }
    return true;
  };
  {
    std::ofstream f;
    if (!open("RowPtr.txt", f)) return false;
    for (int i = 0; i <= g.n; ++i) f << g.row_ptr[i] << "\n";
  }
  {
    std::ofstream f;
    if (!open("ColInd.txt", f)) return false;
    for (int64_t i = 0; i < g.num_edges(); ++i) f << g.col[i] << "\n";
  }
  {
    std::ofstream f;
    if (!open("Values.txt", f)) return false;
    f << std::fixed;
    for (int64_t i = 0; i < g.num_edges(); ++i) f << std::setprecision(6) << g.val[i] << "\n";
  }
  {
    std::ofstream f;
    if (!open("TrueLabels.txt", f)) return false;
    for (int i = 0; i < g.n; ++i) f << i << " " << truth[i] << "\n";
  }
  return true;
}

float mean_edge_weight(const HostGraph &g) {
  if (g.num_edges() == 0) return 0.5f;
  double sum = 0.0;
  int64_t count = 0;
  for (int64_t i = 0; i < g.num_edges(); ++i) {
    if (g.col[i] >= 0) {
      sum += g.val[i];
      ++count;
    }
  }
  return count > 0 ? static_cast<float>(sum / static_cast<double>(count)) : 0.5f;
}

}  // namespace dlp
