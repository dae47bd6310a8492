// Test infrastructure, not product code: IrLP full recompute on a snapshot, the
// reference's validation baseline (src/validation.cu:47-208), on the CPU.
// Every active non-ground-truth vertex is recomputed from the previous buffer
// each iteration; ground-truth and inactive vertices are copied through; the
// ground-truth labels are re-imposed after each iteration; the loop stops at
// the first iteration in which no label moved by more than delta.

#include "oracle.h"
#include "oracle_math.h"

#include <omp.h>

#include <cmath>
#include <vector>

extern "C" int orc_irlp(int n, const int *row_ptr, const int *col_ind, const float *values,
                        const int *status, const int *gt_class, float *labels, float delta,
                        int max_iterations, int threads, int64_t *edge_visits) {
  const int T = threads > 0 ? threads : omp_get_max_threads();
  std::vector<float> a(labels, labels + n), b(labels, labels + n);
  std::vector<float> *old_buf = &a, *new_buf = &b;
  auto skip = [&](int v) { return v < 0 || status[v] == orc::kDeleted; };
  int iters = 0;
  int64_t visits = 0;
  for (int it = 0; it < max_iterations; ++it) {
    const float *src = old_buf->data();
    float *dst = new_buf->data();
    int changed = 0;
    int64_t vis = 0;
#pragma omp parallel for num_threads(T) schedule(dynamic, 1024) reduction(| : changed) reduction(+ : vis)
    for (int u = 0; u < n; ++u) {
      if (gt_class[u] >= 0 || status[u] != orc::kActive) {
        dst[u] = src[u];
        continue;
      }
      const int s = row_ptr[u], len = row_ptr[u + 1] - s;
      vis += len;
      float wa, wl;
      orc::row_sums(col_ind + s, values + s, len, src, skip, wa, wl);
      const float nl = orc::updated_label(wa, wl, src[u]);
      dst[u] = nl;
      if (std::fabs(nl - src[u]) > delta) changed = 1;
    }
    for (int v = 0; v < n; ++v) {
      if (gt_class[v] == 0) dst[v] = 0.0f;
      else if (gt_class[v] == 1) dst[v] = 1.0f;
    }
    std::swap(old_buf, new_buf);
    iters = it + 1;
    visits += vis;
    if (!changed) break;
  }
  for (int v = 0; v < n; ++v) labels[v] = (*old_buf)[v];
  if (edge_visits) *edge_visits = visits;
  return iters;
}
