// Test infrastructure, not product code: CPU oracle of the DynLP per-batch
// update path. See oracle.h for what it restates and who may call it.
//
// Two semantics are carried:
//   ref  - the reference's behaviour (src/dynLP.cu:284-558), including its
//          quirks: the connected-components step hooks the first
//          num_sub_edges *raw* batch edges (src/dynLP.cu:437-440); endpoint
//          marks are clipped to vertex ids below the number of inserted
//          vertices (src/sparsifySubgraph.cu:259-263 with :177-178); a vertex
//          inserted and deleted in the same batch is deleted for that batch
//          only (src/dynLP.cu:118-125 then src/sparsifySubgraph.cu:58-111).
//          The reference reads and writes index -1 of its parent, root and
//          root-to-id arrays (src/connectedComponents.cu:114-115,136,155);
//          those accesses are pinned here as: par[-1] reads -1, the isRoot[-1]
//          write is dropped, rootToId[-1] reads -1. A vertex whose tree reaches
//          -1 therefore gets component -1 and label 0.5.
//   spec - the documented intent: affected set = neighbours of every deleted
//          vertex in the adjacency before the deletion, both endpoints of every
//          new edge and every new non-ground-truth vertex; the sparsified
//          graph is the new-new edges with w > tau and the components are
//          taken on it alone; deletions are permanent.
// Both use the same propagation schedule and arithmetic (oracle_math.h).

#include "oracle.h"
#include "oracle_math.h"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

using orc::kActive;
using orc::kDeleted;
using orc::kGroundTruth;

struct orc_run {
  int n = 0;
  std::vector<int> row_ptr, col;
  std::vector<float> val, truth;
  std::vector<int> batch_map;  // empty: no map
  float tau = 0.5f, delta = 1e-4f;
  int max_iter = 100000, semantics = ORC_SEMANTICS_REF, threads = 1, record = 0;

  std::vector<int8_t> status;  // host-side status (what the reference keeps on the host)
  std::vector<int8_t> gt;      // -1 / 0 / 1
  std::vector<float> labels;
  int fp64 = 0;                 // 1: labels and propagation arithmetic in double;
                                // 2: fp32 run plus a double shadow of each batch's propagation
  std::vector<double> lab64;    // the labels in FP64 mode / the shadow's result
  int shadow_iterations = 0;
  std::string err;

  // scratch
  std::vector<int> arp, acol;  // active CSR of the current batch
  std::vector<float> aval;
  std::vector<int8_t> dev_status;  // status as the batch's kernels see it
  std::vector<uint8_t> affected;
  std::vector<int> local;       // vertex -> position in inserted list, or -1
  std::vector<int> stamp;       // frontier dedup
  int stamp_clock = 0;

  std::vector<std::vector<char>> art;  // artefacts of the last batch
};

namespace {

template <class T>
void set_art(orc_run *r, int which, const std::vector<T> &v) {
  if (!r->record) return;
  auto &a = r->art[which];
  a.resize(v.size() * sizeof(T));
  if (!v.empty()) std::memcpy(a.data(), v.data(), a.size());
}

int nthreads(const orc_run *r) { return r->threads > 0 ? r->threads : omp_get_max_threads(); }

bool in_range(int v, int n) { return v >= 0 && v < n; }

// Rebuilds the active CSR from the full graph: a row is kept for an active
// vertex and filtered to active neighbours, in the full row's (column) order
// (src/dynLP.cu:132-166).
template <class Active>
void rebuild_active(orc_run *r, Active active) {
  const int n = r->n;
  r->arp.assign(static_cast<size_t>(n) + 1, 0);
  std::vector<int> &arp = r->arp;
  const int T = nthreads(r);
#pragma omp parallel for num_threads(T) schedule(static)
  for (int u = 0; u < n; ++u) {
    int c = 0;
    if (active(u))
      for (int k = r->row_ptr[u]; k < r->row_ptr[u + 1]; ++k) {
        const int v = r->col[k];
        if (v >= 0 && active(v)) ++c;
      }
    arp[u + 1] = c;
  }
  for (int u = 0; u < n; ++u) arp[u + 1] += arp[u];
  r->acol.resize(arp[n]);
  r->aval.resize(arp[n]);
#pragma omp parallel for num_threads(T) schedule(static)
  for (int u = 0; u < n; ++u) {
    if (arp[u + 1] == arp[u]) continue;
    int p = arp[u];
    for (int k = r->row_ptr[u]; k < r->row_ptr[u + 1]; ++k) {
      const int v = r->col[k];
      if (v >= 0 && active(v)) {
        r->acol[p] = v;
        r->aval[p++] = r->val[k];
      }
    }
  }
}

// Union-find with path halving over inserted positions plus a sentinel node.
struct DSU {
  std::vector<int> p;
  explicit DSU(int m) : p(m) { std::iota(p.begin(), p.end(), 0); }
  int find(int x) {
    while (p[x] != x) {
      p[x] = p[p[x]];
      x = p[x];
    }
    return x;
  }
  void unite(int a, int b) {
    a = find(a);
    b = find(b);
    if (a != b) p[std::max(a, b)] = std::min(a, b);
  }
};

// Frontier propagation (src/iterativePropagation.cu:241-346) over `labels`
// (float: the reference's arithmetic; double: the FP64 oracle). Two buffers
// that both start at the initial labels; pass k reads buffer k%2 and writes
// buffer (k+1)%2 at frontier vertices only; the result is buffer (passes % 2).
template <class T>
void propagate(orc_run *r, std::vector<T> &labels, std::vector<int> frontier, orc_stats &st,
               std::vector<int> &sizes) {
  std::vector<T> buf[2] = {labels, labels};
  const int T_ = nthreads(r);
  std::vector<std::vector<int>> marks_t(T_);
  auto skip = [&](int v) { return v < 0 || r->dev_status[v] == kDeleted; };
  int passes = 0;
  for (int k = 0; k < r->max_iter; ++k) {
    if (frontier.empty()) break;
    sizes.push_back(static_cast<int>(frontier.size()));
    const T *src = buf[k & 1].data();
    T *dst = buf[(k + 1) & 1].data();
    int64_t edges = 0;
    const int F = static_cast<int>(frontier.size());
#pragma omp parallel num_threads(T_) reduction(+ : edges)
    {
      std::vector<int> &mine = marks_t[omp_get_thread_num()];
      mine.clear();
#pragma omp for schedule(static)
      for (int i = 0; i < F; ++i) {
        const int u = frontier[i];
        const int s = r->arp[u], len = r->arp[u + 1] - s;
        edges += len;
        T nl, old = src[u];
        if constexpr (sizeof(T) == sizeof(float)) {
          float wa, wl;
          orc::row_sums(&r->acol[s], &r->aval[s], len, src, skip, wa, wl);
          nl = orc::updated_label(wa, wl, old);
        } else {
          double wa, wl;
          orc::row_sums64(&r->acol[s], &r->aval[s], len, src, skip, wa, wl);
          nl = orc::updated_label64(wa, wl, old);
        }
        dst[u] = nl;
        if (std::fabs(nl - old) > static_cast<T>(r->delta)) {
          // Mark non-deleted, non-ground-truth neighbours and u itself
          // (src/iterativePropagation.cu:187-217).
          for (int e = s; e < s + len; ++e) {
            const int v = r->acol[e];
            if (v >= 0 && r->dev_status[v] != kDeleted && r->gt[v] < 0) mine.push_back(v);
          }
          if (r->gt[u] < 0) mine.push_back(u);
        }
      }
    }
    st.affected_edges += edges;
    st.frontier_visits += F;
    passes = k + 1;
    // Next frontier: marked, active and not ground truth.
    ++r->stamp_clock;
    std::vector<int> next;
    for (int t = 0; t < T_; ++t)
      for (int v : marks_t[t])
        if (r->stamp[v] != r->stamp_clock) {
          r->stamp[v] = r->stamp_clock;
          if (r->dev_status[v] == kActive && r->gt[v] < 0) next.push_back(v);
        }
    std::sort(next.begin(), next.end());
    frontier.swap(next);
    // A pass with no change marks nothing, so an empty next frontier is the
    // reference's "nothing changed" exit as well.
  }
  st.iterations = passes;
  labels = buf[passes & 1];
  for (size_t v = 0; v < labels.size(); ++v) {  // src/iterativePropagation.cu:224-235
    if (r->gt[v] == 0) labels[v] = 0;
    else if (r->gt[v] == 1) labels[v] = 1;
  }
}

}  // namespace

extern "C" {

orc_run *orc_create(int n, const int *row_ptr, const int *col_ind, const float *values,
                    const float *true_labels, const int *batch_map, float tau, float delta,
                    int max_iterations, int semantics, int threads, int record) {
  if (n <= 0 || !row_ptr) return nullptr;
  orc_run *r = new orc_run();
  r->n = n;
  r->row_ptr.assign(row_ptr, row_ptr + n + 1);
  const int m = r->row_ptr[n];
  r->col.assign(col_ind, col_ind + m);
  r->val.assign(values, values + m);
  if (true_labels) r->truth.assign(true_labels, true_labels + n);
  else r->truth.assign(n, 0.0f);
  if (batch_map) r->batch_map.assign(batch_map, batch_map + n);
  if (tau < 0.0f) {
    // Mean full-graph weight, double accumulation (src/dynLP.cu:90-102,186-190).
    double s = 0.0;
    int64_t c = 0;
    for (int k = 0; k < m; ++k)
      if (r->col[k] >= 0) {
        s += r->val[k];
        ++c;
      }
    tau = c > 0 ? static_cast<float>(s / static_cast<double>(c)) : 0.5f;
  }
  r->tau = tau;
  r->delta = delta;
  r->max_iter = max_iterations;
  r->semantics = semantics;
  r->threads = threads;
  r->record = record;
  r->status.assign(n, kDeleted);
  r->gt.assign(n, -1);
  r->labels.assign(n, 0.5f);
  r->local.assign(n, -1);
  r->stamp.assign(n, 0);
  r->affected.assign(n, 0);
  r->art.resize(ORC_ART_COUNT);
  return r;
}

void orc_destroy(orc_run *r) { delete r; }
float orc_tau(const orc_run *r) { return r->tau; }
const char *orc_error(const orc_run *r) { return r->err.c_str(); }
const float *orc_labels(const orc_run *r) { return r->labels.data(); }
const double *orc_labels64(const orc_run *r) { return r->fp64 ? r->lab64.data() : nullptr; }
int orc_shadow_iterations(const orc_run *r) { return r->shadow_iterations; }

int orc_set_fp64(orc_run *r, int mode) {
  if (!r || mode < 0 || mode > 2) return 1;
  r->fp64 = mode;
  r->lab64.assign(r->labels.begin(), r->labels.end());
  return 0;
}

const void *orc_artefact(const orc_run *r, int which, int64_t *count) {
  if (which < 0 || which >= ORC_ART_COUNT || !r->record) {
    if (count) *count = 0;
    return nullptr;
  }
  const auto &a = r->art[which];
  if (count) *count = static_cast<int64_t>(a.size() / 4);  // every artefact is 4-byte elements
  return a.data();
}

int orc_apply_batch(orc_run *r, int b, const orc_batch_in *in, orc_stats *out) {
  const int n = r->n;
  const bool ref = r->semantics == ORC_SEMANTICS_REF;
  orc_stats st;
  std::memset(&st, 0, sizeof(st));
  st.batch = b;

  // ---- input validation (the reference indexes these ids unchecked) ----
  auto check = [&](const int *ids, int cnt, const char *what) {
    for (int i = 0; i < cnt; ++i)
      if (!in_range(ids[i], n)) {
        r->err = std::string("vertex id out of range in ") + what;
        return false;
      }
    return true;
  };
  if (!check(in->inserted, in->num_inserted, "inserted") || !check(in->gt_ids, in->num_gt, "gt") ||
      !check(in->deleted, in->num_deleted, "deleted") ||
      !check(in->edge_src, in->num_edges, "edge_src") ||
      !check(in->edge_dst, in->num_edges, "edge_dst"))
    return 1;

  const int I = in->num_inserted, E = in->num_edges;

  // ---- step 0: ground-truth classes and labels (src/dynLP.cu:301-305) ----
  for (int i = 0; i < in->num_gt; ++i) {
    const int v = in->gt_ids[i];
    r->gt[v] = in->gt_labels[i] < 0.5f ? 0 : 1;
    r->labels[v] = in->gt_labels[i];
    if (r->fp64) r->lab64[v] = in->gt_labels[i];
  }

  // ---- host status update ----
  std::vector<int8_t> pre_status;  // spec: status before deletions
  if (ref) {
    // delete, then insert, then mark ground truth (src/dynLP.cu:117-130)
    for (int i = 0; i < in->num_deleted; ++i) r->status[in->deleted[i]] = kDeleted;
    for (int i = 0; i < I; ++i) r->status[in->inserted[i]] = kActive;
    for (int i = 0; i < in->num_gt; ++i) r->status[in->gt_ids[i]] = kGroundTruth;
  } else {
    for (int i = 0; i < I; ++i) r->status[in->inserted[i]] = kActive;
    for (int i = 0; i < in->num_gt; ++i) r->status[in->gt_ids[i]] = kGroundTruth;
    pre_status = r->status;
    for (int i = 0; i < in->num_deleted; ++i) r->status[in->deleted[i]] = kDeleted;
  }

  const std::vector<int> &bm = r->batch_map;
  auto active = [&](int v) {
    if (r->status[v] == kDeleted) return false;
    if (!bm.empty() && (bm[v] < 0 || bm[v] > b)) return false;
    return true;
  };
  rebuild_active(r, active);
  if (r->record) {
    set_art(r, ORC_ART_ROW_PTR, r->arp);
    set_art(r, ORC_ART_COL_IND, r->acol);
    set_art(r, ORC_ART_VALUES, r->aval);
    std::vector<int> s32(r->status.begin(), r->status.end());
    set_art(r, ORC_ART_STATUS, s32);
  }

  r->dev_status = r->status;
  std::fill(r->affected.begin(), r->affected.end(), 0);
  for (int i = 0; i < I; ++i) r->local[in->inserted[i]] = i;
  auto is_new = [&](int v) {
    const int p = r->local[v];
    return p >= 0 && p < I && in->inserted[p] == v;
  };

  // ---- step 1a: deletions ----
  if (ref) {
    if (in->num_deleted > 0) {
      // Rows of deleted vertices: mark neighbours, soft-delete the row
      // (src/sparsifySubgraph.cu:58-83). Only a vertex inserted and deleted in
      // this batch still has a row here.
      for (int i = 0; i < in->num_deleted; ++i) {
        const int u = in->deleted[i];
        for (int k = r->arp[u]; k < r->arp[u + 1]; ++k) {
          const int v = r->acol[k];
          if (in_range(v, n)) r->affected[v] = 1;
          r->acol[k] = -1;
        }
        r->dev_status[u] = kDeleted;
      }
      // Entries that point at a deleted vertex (src/sparsifySubgraph.cu:92-111).
      for (int u = 0; u < n; ++u) {
        if (r->dev_status[u] == kDeleted) continue;
        for (int k = r->arp[u]; k < r->arp[u + 1]; ++k) {
          const int v = r->acol[k];
          if (in_range(v, n) && r->dev_status[v] == kDeleted) r->acol[k] = -1;
        }
      }
    }
  } else {
    for (int i = 0; i < in->num_deleted; ++i) {
      const int x = in->deleted[i];
      const bool was_active = pre_status[x] != kDeleted && (bm.empty() || (bm[x] >= 0 && bm[x] <= b));
      if (!was_active) continue;
      for (int k = r->row_ptr[x]; k < r->row_ptr[x + 1]; ++k) {
        const int v = r->col[k];
        if (v >= 0 && active(v)) r->affected[v] = 1;
      }
    }
  }

  // ---- step 1b/2: sparsification, components, label initialisation ----
  std::vector<int> sub_edges, comp_root(I, -1), comp_id(I, -1);
  std::vector<float> init_labels;
  const bool comp_path = ref ? (I > 0 && E > 0) : (I > 0);
  if (comp_path) {
    st.init_branch = 1;
    int kept = 0;
    for (int i = 0; i < E; ++i) {
      const int s = in->edge_src[i], d = in->edge_dst[i];
      const float w = in->edge_weight[i];
      if (w > r->tau && is_new(s) && is_new(d)) {
        ++kept;
        sub_edges.push_back(s);
        sub_edges.push_back(d);
        sub_edges.push_back(d);
        sub_edges.push_back(s);
      }
      if (ref) {
        // Endpoint marks for w > tau, clipped to ids < I (the kernel's numNodes
        // argument is the number of inserted vertices).
        if (w > r->tau) {
          if (s >= 0 && s < I) r->affected[s] = 1;
          if (d >= 0 && d < I) r->affected[d] = 1;
        }
      } else {
        if (active(s)) r->affected[s] = 1;
        if (active(d)) r->affected[d] = 1;
      }
    }
    st.num_sub_edges = 2 * kept;
    if (!ref)
      for (int i = 0; i < I; ++i) {
        const int v = in->inserted[i];
        if (r->gt[v] < 0 && active(v)) r->affected[v] = 1;
      }

    // Components over inserted positions; node I is the -1 sentinel (ref).
    DSU dsu(I + 1);
    int hook_edges = 0;
    bool singleton_by_position = false;
    if (ref) {
      if (st.num_sub_edges > 0) {
        hook_edges = std::min(st.num_sub_edges, E);
        st.hook_truncated = st.num_sub_edges > E ? 1 : 0;
        for (int i = 0; i < hook_edges; ++i) {
          const int s = in->edge_src[i], d = in->edge_dst[i];
          const int a = is_new(s) ? r->local[s] : I;
          const int c = is_new(d) ? r->local[d] : I;
          dsu.unite(a, c);
        }
      } else {
        singleton_by_position = true;  // src/dynLP.cu:441-452
      }
    } else {
      hook_edges = st.num_sub_edges;
      for (size_t k = 0; k < sub_edges.size(); k += 4) dsu.unite(r->local[sub_edges[k]], r->local[sub_edges[k + 1]]);
    }
    st.hook_edges = hook_edges;

    // Canonical root: minimum vertex id of the component; -1 for the sentinel's.
    std::vector<int> min_id(I + 1, -1);
    for (int i = 0; i < I; ++i) {
      const int root = dsu.find(i);
      const int v = in->inserted[i];
      if (min_id[root] < 0 || v < min_id[root]) min_id[root] = v;
    }
    const int sentinel_root = dsu.find(I);
    for (int i = 0; i < I; ++i) {
      const int root = dsu.find(i);
      comp_root[i] = (ref && root == sentinel_root) ? -1 : min_id[root];
    }
    int num_comp = 0;
    if (singleton_by_position) {
      for (int i = 0; i < I; ++i) comp_id[i] = i;
      num_comp = I;
    } else {
      // Sequential ids by ascending root vertex id (src/connectedComponents.cu:264-283).
      std::vector<int> roots;
      for (int i = 0; i < I; ++i)
        if (comp_root[i] >= 0) roots.push_back(comp_root[i]);
      std::sort(roots.begin(), roots.end());
      roots.erase(std::unique(roots.begin(), roots.end()), roots.end());
      num_comp = static_cast<int>(roots.size());
      for (int i = 0; i < I; ++i)
        comp_id[i] = comp_root[i] < 0
                         ? -1
                         : static_cast<int>(std::lower_bound(roots.begin(), roots.end(), comp_root[i]) - roots.begin());
    }
    st.num_components = num_comp;

    // Supernode weights: ground-truth neighbours of each inserted vertex, per
    // component (src/labelInitialization.cu:59-88).
    std::vector<int64_t> w0(std::max(num_comp, 1), 0), w1(std::max(num_comp, 1), 0);
    for (int i = 0; i < I; ++i) {
      const int c = comp_id[i];
      if (c < 0) continue;
      const int u = in->inserted[i];
      for (int k = r->arp[u]; k < r->arp[u + 1]; ++k) {
        const int v = r->acol[k];
        if (v < 0) continue;
        if (r->gt[v] == 0) w0[c] += orc::to_fixed(r->aval[k]);
        else if (r->gt[v] == 1) w1[c] += orc::to_fixed(r->aval[k]);
      }
    }
    // F_u = W1 / (W0 + W1), 0.5 without ground-truth contact
    // (src/labelInitialization.cu:99-142).
    for (int i = 0; i < I; ++i) {
      const int u = in->inserted[i];
      float l;
      if (r->gt[u] == 0) l = 0.0f;
      else if (r->gt[u] == 1) l = 1.0f;
      else if (comp_id[i] < 0) l = 0.5f;
      else {
        const float a = orc::from_fixed(w0[comp_id[i]]);
        const float c = orc::from_fixed(w1[comp_id[i]]);
        const float den = a + c;
        l = den > 1e-10f ? c / den : 0.5f;
      }
      r->labels[u] = l;
      if (r->fp64) {
        double l64 = l;
        if (r->gt[u] < 0 && comp_id[i] >= 0) {
          const double a = static_cast<double>(w0[comp_id[i]]) * (1.0 / 4294967296.0);
          const double c = static_cast<double>(w1[comp_id[i]]) * (1.0 / 4294967296.0);
          const double den = a + c;
          l64 = den > 1e-10 ? c / den : 0.5;
        }
        r->lab64[u] = l64;
      }
    }
  } else if (I > 0) {
    // New vertices without new edges (src/dynLP.cu:482-504): ground truth
    // takes this batch's label, everything else 0.5.
    st.init_branch = 2;
    std::vector<std::pair<int, float>> batch_gt;
    for (int i = 0; i < in->num_gt; ++i) batch_gt.emplace_back(in->gt_ids[i], in->gt_labels[i]);
    for (int i = 0; i < I; ++i) {
      const int v = in->inserted[i];
      float l = 0.5f;
      if (r->gt[v] >= 0)
        for (const auto &p : batch_gt)
          if (p.first == v) l = p.second;
      r->labels[v] = l;
      if (r->fp64) r->lab64[v] = l;
    }
  }
  if (r->record) {
    init_labels.resize(I);
    for (int i = 0; i < I; ++i) init_labels[i] = r->labels[in->inserted[i]];
    set_art(r, ORC_ART_SUB_EDGES, sub_edges);
    set_art(r, ORC_ART_COMP_ROOT, comp_root);
    set_art(r, ORC_ART_COMP_ID, comp_id);
    set_art(r, ORC_ART_INIT_LABELS, init_labels);
    std::vector<int> marks;
    for (int v = 0; v < n; ++v)
      if (r->affected[v]) marks.push_back(v);
    set_art(r, ORC_ART_SEED_MARKS, marks);
  }

  // ---- step 3: frontier propagation (src/iterativePropagation.cu:241-346) ----
  std::vector<int> frontier;
  for (int v = 0; v < n; ++v) {
    if (r->affected[v]) ++st.seed_marks;
    if (r->affected[v] && r->dev_status[v] == kActive && r->gt[v] < 0) frontier.push_back(v);
  }
  st.seed_frontier = static_cast<int>(frontier.size());
  set_art(r, ORC_ART_FRONTIER0, frontier);
  std::vector<int> sizes;
  if (r->fp64 == 1) {
    propagate(r, r->lab64, std::move(frontier), st, sizes);
    for (int v = 0; v < n; ++v) r->labels[v] = static_cast<float>(r->lab64[v]);
  } else {
    if (r->fp64 == 2) {
      // the same batch's propagation in double, from the same state
      r->lab64.assign(r->labels.begin(), r->labels.end());
      orc_stats sh;
      std::memset(&sh, 0, sizeof(sh));
      std::vector<int> sh_sizes;
      propagate(r, r->lab64, frontier, sh, sh_sizes);
      r->shadow_iterations = sh.iterations;
    }
    propagate(r, r->labels, std::move(frontier), st, sizes);
  }
  set_art(r, ORC_ART_FRONTIER_SIZES, sizes);
  set_art(r, ORC_ART_LABELS, r->labels);

  // ---- accuracy over active non-ground-truth vertices (src/dynLP.cu:65-85) ----
  int64_t correct = 0, total = 0;
  for (int v = 0; v < n; ++v) {
    if (r->status[v] == kDeleted || r->status[v] == kGroundTruth) continue;
    const int p = r->labels[v] >= 0.5f ? 1 : 0;
    const int t = r->truth[v] >= 0.5f ? 1 : 0;
    correct += (p == t);
    ++total;
  }
  st.correct = correct;
  st.total = total;
  st.accuracy = total > 0 ? static_cast<float>(correct) / static_cast<float>(total) : 1.0f;
  if (out) *out = st;
  return 0;
}

}  // extern "C"
