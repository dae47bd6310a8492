// Test infrastructure, not product code: arithmetic shared by the oracle's
// propagation and IrLP restatements.
#pragma once

#include <cmath>
#include <cstdint>

namespace orc {

enum : int8_t { kActive = 0, kDeleted = 1, kGroundTruth = 2 };

// Weighted neighbour average in the reference's summation order.
//
// The reference gives each row to a 256-thread block: thread t accumulates row
// entries t, t+256, t+512, ... in that order, weight sum with a plain add and
// weighted label with a multiply-add that nvcc contracts to an FMA
// (src/iterativePropagation.cu:126-136); the 256 partials are then folded by a
// shared-memory tree with strides 128, 64, ..., 1 (:143-150). An entry that is
// skipped leaves its slot at +0. For rows of at most 32 entries the strides
// 128, 64 and 32 only add +0, which leaves every partial unchanged, so the fold
// equals a 32-slot tree with strides 16..1.
template <class Skip>
inline void row_sums(const int *col, const float *val, int len, const float *labels,
                     Skip skip, float &w_all, float &w_label) {
  const int slots = len <= 32 ? 32 : 256;
  float sw[256], sl[256];
  for (int s = 0; s < slots; ++s) sw[s] = sl[s] = 0.0f;
  for (int e = 0; e < len; ++e) {
    const int v = col[e];
    if (skip(v)) continue;
    const int s = e & 255;
    sw[s] = sw[s] + val[e];
    sl[s] = std::fmaf(val[e], labels[v], sl[s]);
  }
  for (int stride = slots / 2; stride > 0; stride >>= 1)
    for (int t = 0; t < stride; ++t) {
      sw[t] = sw[t] + sw[t + stride];
      sl[t] = sl[t] + sl[t + stride];
    }
  w_all = sw[0];
  w_label = sl[0];
}

// The same order in double precision throughout (the FP64 oracle: the same
// schedule with every label, product and sum in double).
template <class Skip>
inline void row_sums64(const int *col, const float *val, int len, const double *labels,
                       Skip skip, double &w_all, double &w_label) {
  const int slots = len <= 32 ? 32 : 256;
  double sw[256], sl[256];
  for (int s = 0; s < slots; ++s) sw[s] = sl[s] = 0.0;
  for (int e = 0; e < len; ++e) {
    const int v = col[e];
    if (skip(v)) continue;
    const int s = e & 255;
    sw[s] = sw[s] + static_cast<double>(val[e]);
    sl[s] = std::fma(static_cast<double>(val[e]), labels[v], sl[s]);
  }
  for (int stride = slots / 2; stride > 0; stride >>= 1)
    for (int t = 0; t < stride; ++t) {
      sw[t] = sw[t] + sw[t + stride];
      sl[t] = sl[t] + sl[t + stride];
    }
  w_all = sw[0];
  w_label = sl[0];
}

// New label from the two sums (src/iterativePropagation.cu:153-168): keep the
// old label when the weight sum is not above 1e-10, clamp to [0, 1]. The
// division is IEEE round-to-nearest (the reference's --use_fast_math build uses
// an approximate division instead; see the parity notes).
inline float updated_label(float w_all, float w_label, float old) {
  float nl = (w_all > 1e-10f) ? (w_label / w_all) : old;
  return std::fmin(std::fmax(nl, 0.0f), 1.0f);
}

inline double updated_label64(double w_all, double w_label, double old) {
  double nl = (w_all > 1e-10) ? (w_label / w_all) : old;
  return std::fmin(std::fmax(nl, 0.0), 1.0);
}

// Supernode weights are summed exactly in 32.32 fixed point, so the sum does
// not depend on the order of the contributions; the reference adds them with
// float atomics whose order varies from run to run
// (src/labelInitialization.cu:76-87).
inline int64_t to_fixed(float w) { return std::llrint(static_cast<double>(w) * 4294967296.0); }
inline float from_fixed(int64_t q) {
  return static_cast<float>(static_cast<double>(q) * (1.0 / 4294967296.0));
}

}  // namespace orc
