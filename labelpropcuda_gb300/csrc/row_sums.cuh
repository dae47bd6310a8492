// Weighted neighbour sums of one row in the reference's summation order.
//
// The reference reduces a row with a 256-thread block: thread t accumulates
// entries t, t+256, t+512, ... (weight with an add, weighted label with a
// multiply-add that nvcc contracts to an FMA), then a shared-memory tree folds
// the 256 partials with strides 128, 64, ..., 1 (src/iterativePropagation.cu:
// 126-150). A skipped entry leaves +0 in its slot.
//
//   group_row_sums<G>: rows of at most 32 entries. Strides 128..32 only add
//     +0 there, so the fold equals a 32-slot tree. Lane l of a G-lane group
//     holds slots l + G*r (r < 32/G); strides 16..G fold in registers, strides
//     G/2..1 by shuffles within the group. The result is identical for any G.
//   warp_row_sums: any length; lane l holds slots l + 32*j (j < 8) and adds
//     every 256th entry into them in order.
//
// `load(e, v, w)` fetches entry e of the row and sets v = -1 for an entry that
// does not count (soft-deleted or pointing at a deleted vertex).
#pragma once

#include <cuda_runtime.h>

namespace dlp {

template <int G, class Load>
__device__ __forceinline__ void group_row_sums(int len, int gl, Load load, const float *labels,
                                               float &w_all, float &w_label, int (&cols)[32 / G]) {
  constexpr int R = 32 / G;
  float sw[R], sl[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int e = gl + G * r;
    sw[r] = 0.0f;
    sl[r] = 0.0f;
    cols[r] = -1;
    if (e < len) {
      int v;
      float w;
      load(e, v, w);
      cols[r] = v;
      if (v >= 0) {
        sw[r] = w;                                // 0 + w
        sl[r] = __fmaf_rn(w, labels[v], 0.0f);    // fma(w, F_v, 0)
      }
    }
  }
#pragma unroll
  for (int half = R / 2; half >= 1; half >>= 1)
#pragma unroll
    for (int r = 0; r < half; ++r) {
      sw[r] = sw[r] + sw[r + half];
      sl[r] = sl[r] + sl[r + half];
    }
  float tw = sw[0], tl = sl[0];
#pragma unroll
  for (int o = G / 2; o >= 1; o >>= 1) {
    tw = tw + __shfl_down_sync(0xffffffffu, tw, o, G);
    tl = tl + __shfl_down_sync(0xffffffffu, tl, o, G);
  }
  w_all = tw;
  w_label = tl;
}

template <class Load>
__device__ __forceinline__ void warp_row_sums(int len, int lane, Load load, const float *labels,
                                              float &w_all, float &w_label) {
  float sw[8], sl[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) sw[j] = sl[j] = 0.0f;
  for (int p = 0; p < len; p += 256) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int e = p + j * 32 + lane;
      if (e < len) {
        int v;
        float w;
        load(e, v, w);
        if (v >= 0) {
          sw[j] = sw[j] + w;
          sl[j] = __fmaf_rn(w, labels[v], sl[j]);
        }
      }
    }
  }
#pragma unroll
  for (int half = 4; half >= 1; half >>= 1)
#pragma unroll
    for (int j = 0; j < half; ++j) {
      sw[j] = sw[j] + sw[j + half];
      sl[j] = sl[j] + sl[j + half];
    }
  float tw = sw[0], tl = sl[0];
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    tw = tw + __shfl_down_sync(0xffffffffu, tw, o);
    tl = tl + __shfl_down_sync(0xffffffffu, tl, o);
  }
  w_all = tw;
  w_label = tl;
}

}  // namespace dlp
