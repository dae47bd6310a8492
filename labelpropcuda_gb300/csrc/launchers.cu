// The reference's five step launchers on caller-owned device arrays in the
// reference's layout (packed CSR with separate colInd / values, int32 status,
// gtClass and isAffected arrays). C ABI group 3 in dlp_gb300.h.
//
// Each launcher keeps the reference's argument meaning and its outputs,
// including the soft-delete (-1) entries and the final isAffected state, but
// runs as GB300 kernels: group-per-row walks instead of a 256-thread block per
// row, a single cooperative kernel for the whole Shiloach-Vishkin loop and for
// the whole propagation loop (no host round trip per round), and stream-ordered
// temporaries (cudaMallocAsync) instead of cudaMalloc/cudaFree per round. They
// synchronise the stream only to return a scalar through a pointer
// (numSubEdges, numComponents, iterationsUsed), as the reference's int&
// outputs require.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "row_sums.cuh"

namespace dlp {
namespace ref_layout {
namespace {

// Division of the label updates in the launchers (dlp_set_launcher_arithmetic).
std::atomic<int> g_launcher_arith{DLP_ARITH_IEEE};

constexpr int kBlock = 256;
constexpr int kGroup = 8;               // lanes per row in the row walks
constexpr int kMaxHookRounds = 100;     // src/connectedComponents.cu:209
constexpr int kNarrowMax = 32;
constexpr int kChunkBits = 1024;        // rank bitmap chunk

__device__ __forceinline__ bool in_range(int v, int n) {
  return static_cast<unsigned>(v) < static_cast<unsigned>(n);
}

int grid_for(long long items, int per_block) {
  long long g = (items + per_block - 1) / per_block;
  return static_cast<int>(std::max<long long>(1, std::min<long long>(g, 152LL * 32)));
}

template <class T>
int tmp_alloc(T **p, size_t count, cudaStream_t s) {
  DLP_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void **>(p), std::max<size_t>(count, 1) * sizeof(T), s));
  return DLP_OK;
}

// ------------------------------------------------------- mark deletions ----
// src/sparsifySubgraph.cu:58-83: neighbours of each deleted vertex's row are
// affected, the row is soft-deleted, the vertex becomes DELETED.
__global__ void mark_deleted_rows(const int *row_ptr, int *col, int *status, int *affected,
                                  const int *deleted, int count, int n) {
  const int lane = threadIdx.x & 31, gl = lane & (kGroup - 1);
  const int group = (blockIdx.x * blockDim.x + threadIdx.x) / kGroup;
  const int groups = gridDim.x * blockDim.x / kGroup;
  for (int i = group; i < count; i += groups) {
    const int u = deleted[i];
    if (!in_range(u, n)) continue;
    const int rs = row_ptr[u], re = row_ptr[u + 1];
    for (int e = rs + gl; e < re; e += kGroup) {
      const int v = col[e];
      if (in_range(v, n)) atomicMax(&affected[v], 1);
      col[e] = -1;
    }
    if (gl == 0) status[u] = kDeleted;
  }
}

// src/sparsifySubgraph.cu:92-111: entries pointing at a DELETED vertex.
__global__ void clean_incoming(const int *row_ptr, int *col, const int *status, int n) {
  const int lane = threadIdx.x & 31, gl = lane & (kGroup - 1);
  const int group = (blockIdx.x * blockDim.x + threadIdx.x) / kGroup;
  const int groups = gridDim.x * blockDim.x / kGroup;
  for (int u = group; u < n; u += groups) {
    if (status[u] == kDeleted) continue;
    const int rs = row_ptr[u], re = row_ptr[u + 1];
    for (int e = rs + gl; e < re; e += kGroup) {
      const int v = col[e];
      if (in_range(v, n) && status[v] == kDeleted) col[e] = -1;
    }
  }
}

// ---------------------------------------------------------- sparsify -------
struct SparsifyArgs {
  const int *src, *dst;
  const float *w;
  int m;
  const int *is_new;
  int n;
  float tau;
};

__device__ __forceinline__ bool kept_edge(const SparsifyArgs &a, int i, int &u, int &v, float &w, bool &bad) {
  u = a.src[i];
  v = a.dst[i];
  w = a.w[i];
  if (!in_range(u, a.n) || !in_range(v, a.n)) {
    bad = true;
    return false;
  }
  return a.is_new[u] && a.is_new[v] && w > a.tau;
}

// Per-block count of kept edges (src/sparsifySubgraph.cu:119-136).
__global__ void sparsify_count(SparsifyArgs a, int *block_counts, int *total, int *err) {
  __shared__ int s_count;
  if (threadIdx.x == 0) s_count = 0;
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool bad = false;
  int u, v;
  float w;
  const bool k = i < a.m && kept_edge(a, i, u, v, w, bad);
  const unsigned m = __ballot_sync(0xffffffffu, k);
  if ((threadIdx.x & 31) == 0 && m) atomicAdd(&s_count, __popc(m));
  if (bad) atomicExch(err, DLP_ERR_INVALID_ARGUMENT);
  __syncthreads();
  if (threadIdx.x == 0) {
    block_counts[blockIdx.x] = s_count;
    if (s_count) atomicAdd(total, 2 * s_count);
  }
}

// Writes kept edges in raw order (both directions) and the clipped endpoint
// marks (src/sparsifySubgraph.cu:144-179 with numNodes = numInserted,
// :259-263).
__global__ void sparsify_build(SparsifyArgs a, const int *block_counts, int *affected, int mark_limit,
                               int *sub_col, float *sub_val) {
  __shared__ int s_warp[kBlock / 32];
  __shared__ int s_base;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // this block's first slot: the kept edges of the blocks before it, summed
  // by the whole block (one load per thread per 1024 blocks, not a serial walk)
  {
    int part = 0;
    for (int q = threadIdx.x; q < static_cast<int>(blockIdx.x); q += blockDim.x) part += block_counts[q];
    part = __reduce_add_sync(0xffffffffu, part);
    if (lane == 0) s_warp[wid] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
      int b = 0;
      for (int q = 0; q < kBlock / 32; ++q) b += s_warp[q];
      s_base = b;
    }
    __syncthreads();
  }
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool bad = false;
  int u = 0, v = 0;
  float w = 0.0f;
  const bool k = i < a.m && kept_edge(a, i, u, v, w, bad);
  const unsigned m = __ballot_sync(0xffffffffu, k);
  if (lane == 0) s_warp[wid] = __popc(m);
  __syncthreads();
  if (k) {
    int pos = s_base;
    for (int q = 0; q < wid; ++q) pos += s_warp[q];
    pos += __popc(m & ((1u << lane) - 1u));
    sub_col[2 * pos] = v;
    sub_col[2 * pos + 1] = u;
    sub_val[2 * pos] = w;
    sub_val[2 * pos + 1] = w;
  }
  if (i < a.m && !bad && w > a.tau) {
    if (u >= 0 && u < mark_limit) atomicMax(&affected[u], 1);
    if (v >= 0 && v < mark_limit) atomicMax(&affected[v], 1);
  }
}

// ------------------------------------------------- connected components ----
__global__ void cc_validate_init(const int *es, const int *ed, int m, const int *ins, int I, int n, int *par,
                                 int *err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
  for (int i = t; i < m; i += nt)
    if (!in_range(es[i], n) || !in_range(ed[i], n)) atomicExch(err, DLP_ERR_INVALID_ARGUMENT);
  for (int i = t; i < I; i += nt) {
    const int v = ins[i];
    if (!in_range(v, n)) atomicExch(err, DLP_ERR_INVALID_ARGUMENT);
    else par[v] = v;  // src/connectedComponents.cu:64-71
  }
}

struct CcArgs {
  const int *es, *ed;
  int m;
  const int *ins;
  int I;
  int *par;
  int *flags;  // [kMaxHookRounds] hook-changed, [kMaxHookRounds] = rounds used
  GridBarrier *bar;
  int *err;
  unsigned long long timeout_ns;
};

// Hook (atomicMin of the larger root under the smaller, src/connectedComponents.cu:79-100)
// and full pointer jumping (:108-121) until a hook pass changes nothing. par
// holds -1 for vertices that are not inserted, as in the reference.
__global__ void __launch_bounds__(kBlock) cc_sv_kernel(CcArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
  if (ld_relaxed_i32(a.err) != 0) return;
  int rounds = 0;
  for (int r = 0; r < kMaxHookRounds; ++r) {
    bool changed = false;
    for (int i = t; i < a.m; i += nt) {
      const int ru = a.par[a.es[i]];
      const int rv = a.par[a.ed[i]];
      if (ru != rv) {
        const int hi = max(ru, rv), lo = min(ru, rv);
        if (atomicMin(&a.par[hi], lo) != lo) changed = true;
      }
    }
    if (__any_sync(0xffffffffu, changed) && (threadIdx.x & 31) == 0) a.flags[r] = 1;
    if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
    for (int i = t; i < a.I; i += nt) {
      const int v = a.ins[i];
      int p = a.par[v];
      while (p >= 0) {  // par[-1] reads as -1
        const int q = a.par[p];
        if (q == p) break;
        p = q;
      }
      a.par[v] = p;
    }
    if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
    rounds = r + 1;
    if (ld_relaxed_i32(&a.flags[r]) == 0) break;
  }
  if (t == 0) a.flags[kMaxHookRounds] = rounds;
}

// Root bitmap (src/connectedComponents.cu:129-137; the isRoot[-1] write of a
// vertex whose root is -1 is dropped).
__global__ void cc_mark_roots(const int *par, const int *ins, int I, unsigned *bits) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
  for (int i = t; i < I; i += nt) {
    const int r = par[ins[i]];
    if (r >= 0) atomicOr(&bits[r >> 5], 1u << (r & 31));
  }
}

// Exclusive prefix of set bits per 1024-bit chunk (one block).
__global__ void cc_chunk_scan(const unsigned *bits, int words, int *chunk_prefix, int chunks, int *total) {
  __shared__ int s_carry;
  __shared__ int s_vals[1024];
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int base = 0; base < chunks; base += blockDim.x) {
    const int c = base + threadIdx.x;
    int cnt = 0;
    if (c < chunks)
      for (int wd = c * (kChunkBits / 32); wd < min(words, (c + 1) * (kChunkBits / 32)); ++wd) cnt += __popc(bits[wd]);
    s_vals[threadIdx.x] = cnt;
    __syncthreads();
    for (int o = 1; o < blockDim.x; o <<= 1) {  // inclusive Hillis-Steele scan
      const int add = threadIdx.x >= o ? s_vals[threadIdx.x - o] : 0;
      __syncthreads();
      s_vals[threadIdx.x] += add;
      __syncthreads();
    }
    if (c < chunks) chunk_prefix[c] = s_carry + s_vals[threadIdx.x] - cnt;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) s_carry += s_vals[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = s_carry;
}

// componentId[v] = rank of v's root among roots in ascending vertex order
// (src/connectedComponents.cu:264-283); -1 when the root is -1.
__global__ void cc_assign(const int *par, const int *ins, int I, const unsigned *bits, const int *chunk_prefix,
                          int *comp) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
  for (int i = t; i < I; i += nt) {
    const int v = ins[i];
    const int r = par[v];
    if (r < 0) {
      comp[v] = -1;
      continue;
    }
    const int word = r >> 5;
    const int c = r / kChunkBits;
    int rank = chunk_prefix[c];
    for (int wd = c * (kChunkBits / 32); wd < word; ++wd) rank += __popc(bits[wd]);
    rank += __popc(bits[word] & ((1u << (r & 31)) - 1u));
    comp[v] = rank;
  }
}

// ---------------------------------------------------- label init ----------
// src/labelInitialization.cu:59-88, with exact fixed-point sums.
__global__ void init_accumulate(const int *row_ptr, const int *col, const float *val, const int *comp,
                                int num_comp, const int *gt, const int *ins, int I, int n, long long *acc) {
  const int lane = threadIdx.x & 31, gl = lane & (kGroup - 1);
  const int group = (blockIdx.x * blockDim.x + threadIdx.x) / kGroup;
  const int groups = gridDim.x * blockDim.x / kGroup;
  const int rounds = (I + groups - 1) / groups;
  for (int k = 0; k < rounds; ++k) {
    const int i = group + k * groups;
    int c = -1, rs = 0, re = 0;
    if (i < I) {
      const int u = ins[i];
      if (in_range(u, n)) {
        c = comp[u];
        if (c >= num_comp) c = -1;  // out-of-range ids are treated as no component
        if (c >= 0) {
          rs = row_ptr[u];
          re = row_ptr[u + 1];
        }
      }
    }
    long long q0 = 0, q1 = 0;
    for (int e = rs + gl; e < re; e += kGroup) {
      const int v = col[e];
      if (!in_range(v, n)) continue;
      const int g = gt[v];
      if (g == 0) q0 += to_fixed(val[e]);
      else if (g == 1) q1 += to_fixed(val[e]);
    }
#pragma unroll
    for (int o = kGroup / 2; o > 0; o >>= 1) {
      q0 += __shfl_down_sync(0xffffffffu, q0, o, kGroup);
      q1 += __shfl_down_sync(0xffffffffu, q1, o, kGroup);
    }
    if (gl == 0 && c >= 0) {
      if (q0) atomicAdd(reinterpret_cast<unsigned long long *>(&acc[2 * c]), static_cast<unsigned long long>(q0));
      if (q1) atomicAdd(reinterpret_cast<unsigned long long *>(&acc[2 * c + 1]), static_cast<unsigned long long>(q1));
    }
  }
}

// src/labelInitialization.cu:99-142.
__global__ void init_labels(float *labels, const int *comp, int num_comp, const int *gt, const long long *acc,
                            const int *ins, int I, int n, int fast_div) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
  for (int i = t; i < I; i += nt) {
    const int u = ins[i];
    if (!in_range(u, n)) continue;
    const int g = gt[u];
    if (g == 0) { labels[u] = 0.0f; continue; }
    if (g == 1) { labels[u] = 1.0f; continue; }
    const int c = comp[u];
    if (c < 0 || c >= num_comp) { labels[u] = 0.5f; continue; }
    const float w0 = from_fixed(acc[2 * c]);
    const float w1 = from_fixed(acc[2 * c + 1]);
    const float den = w0 + w1;
    labels[u] = den > 1e-10f ? quotient(w1, den, fast_div) : 0.5f;
  }
}

// ------------------------------------------------------- propagation -------
struct PropArgs {
  const int *row_ptr, *col;
  const float *val;
  float *labels, *buffer;
  const int *status, *gt;
  int *affected;
  int n;
  float delta;
  int max_iter;
  unsigned *stamp;     // n, zeroed
  int *lists;          // 3n
  int *counts;         // [3][2]
  int *out;            // [0] passes, [1] last mark stamp, [2] next pass after a block-0 stint
  GridBarrier *bar;
  int *err;
  unsigned long long timeout_ns;
  int fast_div;        // the division of the label updates (dlp_set_launcher_arithmetic)
};

// Frontier loop of src/iterativePropagation.cu:274-327 in one cooperative
// launch; per pass, the frontier is the set of vertices marked in the previous
// pass that are ACTIVE and not ground truth.
template <int G>
__global__ void __launch_bounds__(kBlock) prop_kernel(PropArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31, gwarp = t >> 5, nwarps = nt >> 5;
  const int n = a.n;
  if (ld_relaxed_i32(a.err) != 0) return;
  auto append = [&](bool pred, int v, int set) {
    bool wide = false;
    if (pred) wide = a.row_ptr[v + 1] - a.row_ptr[v] > kNarrowMax;
    int *list = a.lists + static_cast<size_t>(set) * n;
    warp_append(pred && !wide, v, list, &a.counts[2 * set]);
    warp_append_back(pred && wide, v, list, n, &a.counts[2 * set + 1]);
  };
  // seed: src/iterativePropagation.cu:63-78
  for (int base = gwarp * 32; base < n; base += nwarps * 32) {
    const int v = base + lane;
    const bool ok = v < n && a.affected[v] == 1 && a.status[v] == kActive && a.gt[v] < 0;
    append(ok, v, 0);
  }
  if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;

  constexpr int GPW = 32 / G;
  const int grp = lane / G, gl = lane & (G - 1);
  // The rows of pass k (nn narrow, nw wide in list k % 3) by the warps
  // [w0, w0 + nws) of the launch; marks go to list (k + 1) % 3.
  auto rows = [&](int k, int nn, int nw, int w0, int nws) {
    const int set = k % 3;
    const float *src = (k & 1) ? a.buffer : a.labels;
    float *dst = (k & 1) ? a.labels : a.buffer;
    const unsigned stamp = static_cast<unsigned>(k) + 1u;
    const int nset = (k + 1) % 3;
    const int *cur = a.lists + static_cast<size_t>(set) * n;
    auto mark = [&](bool cand, int v) {
      bool fresh = false;
      if (cand) fresh = atomicMax(&a.stamp[v], stamp) < stamp;
      append(fresh && a.status[v] == kActive && a.gt[v] < 0, v, nset);
    };
    for (int base = w0 * GPW; base < nn; base += nws * GPW) {
      const int item = base + grp;
      const bool valid = item < nn;
      int u = 0, rs = 0, len = 0;
      if (valid) {
        u = cur[item];
        rs = a.row_ptr[u];
        len = a.row_ptr[u + 1] - rs;
      }
      auto load = [&](int e, int &v, float &w) {
        v = a.col[rs + e];
        w = a.val[rs + e];
        if (v >= 0 && a.status[v] == kDeleted) v = -1;
      };
      float tw, tl;
      int cols[32 / G];
      group_row_sums<G>(len, gl, load, src, tw, tl, cols);
      int changed = 0;
      if (valid && gl == 0) {
        const float old = src[u];
        const float nl = updated_label(tw, tl, old, a.fast_div);
        dst[u] = nl;
        changed = fabsf(nl - old) > a.delta;
      }
      changed = __shfl_sync(0xffffffffu, changed, 0, G);
#pragma unroll
      for (int r = 0; r < 32 / G; ++r) mark(changed && cols[r] >= 0 && a.gt[cols[r]] < 0, cols[r]);
      mark(changed && gl == 0 && a.gt[u] < 0, u);
    }
    for (int wi = w0; wi < nw; wi += nws) {
      const int u = cur[n - 1 - wi];
      const int rs = a.row_ptr[u], len = a.row_ptr[u + 1] - rs;
      auto load = [&](int e, int &v, float &w) {
        v = a.col[rs + e];
        w = a.val[rs + e];
        if (v >= 0 && a.status[v] == kDeleted) v = -1;
      };
      float tw, tl;
      warp_row_sums(len, lane, load, src, tw, tl);
      int changed = 0;
      if (lane == 0) {
        const float old = src[u];
        const float nl = updated_label(tw, tl, old, a.fast_div);
        dst[u] = nl;
        changed = fabsf(nl - old) > a.delta;
      }
      changed = __shfl_sync(0xffffffffu, changed, 0);
      if (changed) {
        for (int e0 = 0; e0 < len; e0 += 32) {
          const int e = e0 + lane;
          int v = e < len ? a.col[rs + e] : -1;
          if (v >= 0 && a.status[v] == kDeleted) v = -1;
          mark(v >= 0 && a.gt[v] < 0, v);
        }
        mark(lane == 0 && a.gt[u] < 0, u);
      }
    }
  };
  // A frontier of narrow rows that one block takes in one round runs on
  // block 0 alone, pass after pass with block barriers, while the other
  // blocks wait at the next grid barrier: a pass then costs a block barrier
  // instead of a grid barrier. The stint ends when the frontier empties,
  // outgrows one round or gets a wide row, at maxIter, or after 100 ms (the
  // waiting blocks' barrier has a 2 s limit); block 0 publishes the next pass.
  constexpr int kSmallFront = kBlock / G;
  __shared__ int s_stop;
  int k = 0;
  for (;;) {
    const int set = k % 3;
    const int nn = ld_relaxed_i32(&a.counts[2 * set]);
    const int nw = ld_relaxed_i32(&a.counts[2 * set + 1]);
    if (nn + nw == 0 || k >= a.max_iter) break;
    if (nw == 0 && nn <= kSmallFront) {
      if (blockIdx.x == 0) {
        const int warp = threadIdx.x >> 5;
        const uint64_t t_start = global_timer_ns();
        if (threadIdx.x == 0) s_stop = 0;
        __syncthreads();
        for (;;) {
          const int cs = k % 3;
          const int cn = ld_relaxed_i32(&a.counts[2 * cs]);
          const int cw = ld_relaxed_i32(&a.counts[2 * cs + 1]);
          // the same decision in every thread: all inputs were written
          // before the last block barrier
          if (cn + cw == 0 || cw != 0 || cn > kSmallFront || k >= a.max_iter || s_stop) break;
          if (threadIdx.x == 0) {
            a.counts[2 * ((k + 2) % 3)] = 0;
            a.counts[2 * ((k + 2) % 3) + 1] = 0;
            if ((k & 15) == 15 && global_timer_ns() - t_start > 100000000ull) s_stop = 1;
          }
          rows(k, cn, 0, warp, kBlock / 32);
          __syncthreads();
          ++k;
        }
        if (threadIdx.x == 0) a.out[2] = k;
      }
      if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
      k = ld_relaxed_i32(&a.out[2]);
      continue;
    }
    if (t == 0) {
      a.counts[2 * ((k + 2) % 3)] = 0;
      a.counts[2 * ((k + 2) % 3) + 1] = 0;
    }
    rows(k, nn, nw, gwarp, nwarps);
    if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
    ++k;
  }
  // final labels in the primary array, ground truth enforced
  // (src/iterativePropagation.cu:330-339); isAffected holds the last pass's marks
  for (int v = t; v < n; v += nt) {
    float l = (k & 1) ? a.buffer[v] : a.labels[v];
    const int g = a.gt[v];
    if (g == 0) l = 0.0f;
    else if (g == 1) l = 1.0f;
    a.labels[v] = l;
    if (k > 0) a.affected[v] = a.stamp[v] == static_cast<unsigned>(k) ? 1 : 0;
  }
  if (t == 0) a.out[0] = k;
}

// ------------------------------------------------------------------ IrLP ---
struct IrlpArgs {
  const int *row_ptr, *col;
  const float *val;
  float *labels, *buffer;
  const int *status, *gt;
  int n;
  float delta;
  int max_iter;
  int *flags;  // [3] changed per pass (triple buffered), [4] passes
  GridBarrier *bar;
  int *err;
  unsigned long long timeout_ns;
};

// src/validation.cu:47-139 and :169-197 in one cooperative launch: all
// vertices every pass; ground truth and inactive vertices are copied through
// (ground truth re-imposed as 0/1); stop after a pass with no move > delta.
__global__ void __launch_bounds__(kBlock) irlp_kernel(IrlpArgs a) {
  constexpr int G = 8;
  const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31, gwarp = t >> 5, nwarps = nt >> 5;
  const int grp = lane / G, gl = lane & (G - 1);
  if (ld_relaxed_i32(a.err) != 0) return;
  int k = 0;
  for (; k < a.max_iter; ++k) {
    const float *src = (k & 1) ? a.buffer : a.labels;
    float *dst = (k & 1) ? a.labels : a.buffer;
    // flags[k%3] is read right after this pass's barrier; flags[(k+1)%3] was
    // last read after barrier k-2, which every block has left
    if (t == 0) a.flags[(k + 1) % 3] = 0;
    bool changed = false;
    for (int base = gwarp * (32 / G); base < a.n; base += nwarps * (32 / G)) {
      const int u = base + grp;
      const bool valid = u < a.n;
      bool compute = false;
      int rs = 0, len = 0;
      if (valid) {
        compute = a.gt[u] < 0 && a.status[u] == kActive;
        if (compute) {
          rs = a.row_ptr[u];
          len = a.row_ptr[u + 1] - rs;
        }
      }
      // one uniform path per warp: long rows fall back to a serial walk by
      // the group (still in the reference's slot order via warp_row_sums below)
      const bool any_long = __any_sync(0xffffffffu, len > kNarrowMax);
      float tw = 0.0f, tl = 0.0f;
      auto load = [&](int e, int &v, float &w) {
        v = a.col[rs + e];
        w = a.val[rs + e];
        if (v >= 0 && a.status[v] == kDeleted) v = -1;
      };
      if (!any_long) {
        int cols[32 / G];
        group_row_sums<G>(len, gl, load, src, tw, tl, cols);
      } else {
        // each group's row in turn, by the whole warp
        for (int q = 0; q < 32 / G; ++q) {
          const int uq = __shfl_sync(0xffffffffu, u, q * G);
          const int rq = __shfl_sync(0xffffffffu, rs, q * G);
          const int lq = __shfl_sync(0xffffffffu, len, q * G);
          auto lq_load = [&](int e, int &v, float &w) {
            v = a.col[rq + e];
            w = a.val[rq + e];
            if (v >= 0 && a.status[v] == kDeleted) v = -1;
          };
          float w1, l1;
          warp_row_sums(lq, lane, lq_load, src, w1, l1);
          (void)uq;
          const float w1b = __shfl_sync(0xffffffffu, w1, 0);
          const float l1b = __shfl_sync(0xffffffffu, l1, 0);
          if (grp == q) {
            tw = w1b;
            tl = l1b;
          }
        }
      }
      if (valid && gl == 0) {
        if (!compute) {
          const int g = a.gt[u];
          dst[u] = g == 0 ? 0.0f : (g == 1 ? 1.0f : src[u]);
        } else {
          const float old = src[u];
          const float nl = updated_label(tw, tl, old);
          dst[u] = nl;
          if (fabsf(nl - old) > a.delta) changed = true;
        }
      }
    }
    if (__any_sync(0xffffffffu, changed) && lane == 0) a.flags[k % 3] = 1;
    if (!grid_sync(a.bar, a.err, a.timeout_ns)) return;
    if (ld_relaxed_i32(&a.flags[k % 3]) == 0) {
      ++k;
      break;
    }
  }
  // the result is the buffer written last; make it the primary array
  if (k & 1)
    for (int v = t; v < a.n; v += nt) a.labels[v] = a.buffer[v];
  if (t == 0) a.flags[4] = k;
}

const void *prop_kernel_ptr(int lanes) {
  switch (lanes) {
    case 4: return reinterpret_cast<const void *>(&prop_kernel<4>);
    case 16: return reinterpret_cast<const void *>(&prop_kernel<16>);
    case 32: return reinterpret_cast<const void *>(&prop_kernel<32>);
    default: return reinterpret_cast<const void *>(&prop_kernel<8>);
  }
}

int coop_grid(const void *kernel) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0) != cudaSuccess || per_sm <= 0) {
    cudaGetLastError();
    return -1;
  }
  return sms * per_sm;
}

}  // namespace
}  // namespace ref_layout
}  // namespace dlp

using namespace dlp::ref_layout;

// ---------------------------------------------------------------------------
// Scratch of dlp_iterative_propagation_noalloc: the frontier stamps, the three
// frontier lists, the counters and the grid barrier of one propagation call on
// a graph of at most kNoAllocMaxNodes vertices (16 MiB + 1 KiB). It is a
// file-scope device array, so it exists on every GPU that loads this library,
// from module load until the process exits, whether or not the entry point is
// ever called.
namespace {
constexpr int kNoAllocMaxNodes = 1 << 20;
struct NoAllocScratch {
  unsigned stamp[kNoAllocMaxNodes];
  int lists[3 * kNoAllocMaxNodes];
  int small[16];
  dlp::GridBarrier bar;
};
}  // namespace

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

namespace {
// The array's device address, looked up once per device (the host-side name
// of a __device__ variable is not a device address). Fixed table: no heap use.
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
NoAllocScratch *g_noalloc_addr[kNoAllocMaxDevices] = {};

int noalloc_scratch(NoAllocScratch **out) {
  int dev = -1;
  DLP_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "device ordinal too large");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return dlp::cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
    g_noalloc_addr[dev] = static_cast<NoAllocScratch *>(p);
  }
  *out = g_noalloc_addr[dev];
  return DLP_OK;
}
}  // namespace

extern "C" {

int dlp_set_launcher_arithmetic(int arithmetic) {
  dlp::clear_error();
  if (arithmetic != DLP_ARITH_IEEE && arithmetic != DLP_ARITH_REFERENCE_FAST_MATH)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "arithmetic must be DLP_ARITH_IEEE or DLP_ARITH_REFERENCE_FAST_MATH");
  g_launcher_arith.store(arithmetic);
  return DLP_OK;
}

int dlp_mark_deletions(int *d_row_ptr, int *d_col_ind, int *d_vertex_status, int *d_is_affected,
                       const int *d_deleted_nodes, int num_deleted, int num_nodes, void *stream) {
  dlp::clear_error();
  if (num_deleted == 0) return DLP_OK;  // src/sparsifySubgraph.cu:188
  if (num_deleted < 0 || num_nodes <= 0 || !d_row_ptr || !d_vertex_status || !d_is_affected || !d_deleted_nodes)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "invalid arguments to dlp_mark_deletions");
  DLP_TRY(dlp::require_device());
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  mark_deleted_rows<<<grid_for(static_cast<long long>(num_deleted) * kGroup, kBlock), kBlock, 0, s>>>(
      d_row_ptr, d_col_ind, d_vertex_status, d_is_affected, d_deleted_nodes, num_deleted, num_nodes);
  DLP_CUDA_TRY(cudaGetLastError());
  clean_incoming<<<grid_for(static_cast<long long>(num_nodes) * kGroup, kBlock), kBlock, 0, s>>>(
      d_row_ptr, d_col_ind, d_vertex_status, num_nodes);
  DLP_CUDA_TRY(cudaGetLastError());
  return DLP_OK;
}

int dlp_build_sparsified_subgraph(int *d_row_ptr, int *d_col_ind, float *d_values, int *d_is_affected,
                                  const int *d_vertex_status, const int *d_new_edge_src, const int *d_new_edge_dst,
                                  const float *d_new_edge_weight, int num_new_edges, const int *d_inserted_nodes,
                                  int num_inserted, const int *d_is_new_vertex, float tau, int *d_sub_row_ptr,
                                  int *d_sub_col_ind, float *d_sub_values, int *num_sub_nodes, int *num_sub_edges,
                                  void *stream) {
  (void)d_row_ptr;
  (void)d_col_ind;
  (void)d_values;
  (void)d_vertex_status;
  (void)d_inserted_nodes;
  (void)d_sub_row_ptr;  // never written by the reference either
  dlp::clear_error();
  if (!num_sub_nodes || !num_sub_edges) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null outputs");
  *num_sub_nodes = num_inserted;
  *num_sub_edges = 0;
  if (num_new_edges == 0) return DLP_OK;  // src/sparsifySubgraph.cu:213-217
  if (num_new_edges < 0 || !d_new_edge_src || !d_new_edge_dst || !d_new_edge_weight || !d_is_new_vertex ||
      !d_is_affected || !d_sub_col_ind || !d_sub_values)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "invalid arguments to dlp_build_sparsified_subgraph");
  DLP_TRY(dlp::require_device());
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // The reference's signature carries no vertex count, so endpoints can only be
  // checked for being non-negative; the endpoint marks are clipped to ids below
  // numInserted, the numNodes the reference passes there (src/sparsifySubgraph.cu:263).
  const int n_guard = 0x7fffffff;
  const int blocks = (num_new_edges + kBlock - 1) / kBlock;
  int *blk = nullptr, *scal = nullptr;
  DLP_TRY(tmp_alloc(&blk, blocks, s));
  DLP_TRY(tmp_alloc(&scal, 2, s));
  DLP_CUDA_TRY(cudaMemsetAsync(scal, 0, 2 * sizeof(int), s));
  SparsifyArgs a{d_new_edge_src, d_new_edge_dst, d_new_edge_weight, num_new_edges, d_is_new_vertex, n_guard, tau};
  sparsify_count<<<blocks, kBlock, 0, s>>>(a, blk, scal, scal + 1);
  DLP_CUDA_TRY(cudaGetLastError());
  int host[2] = {0, 0};
  DLP_CUDA_TRY(cudaMemcpyAsync(host, scal, sizeof(host), cudaMemcpyDeviceToHost, s));
  DLP_CUDA_TRY(cudaStreamSynchronize(s));
  if (host[1] != 0) {
    cudaFreeAsync(blk, s);
    cudaFreeAsync(scal, s);
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "edge endpoint out of range");
  }
  *num_sub_edges = host[0];
  sparsify_build<<<blocks, kBlock, 0, s>>>(a, blk, d_is_affected, num_inserted, d_sub_col_ind, d_sub_values);
  DLP_CUDA_TRY(cudaGetLastError());
  DLP_CUDA_TRY(cudaFreeAsync(blk, s));
  DLP_CUDA_TRY(cudaFreeAsync(scal, s));
  return DLP_OK;
}

int dlp_connected_components(const int *d_edge_src, const int *d_edge_dst, int num_edges,
                             const int *d_inserted_nodes, int num_inserted, int *d_component_id,
                             int *num_components, int num_nodes, void *stream) {
  dlp::clear_error();
  if (!num_components) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null num_components");
  if (num_inserted == 0) {  // src/connectedComponents.cu:167-170
    *num_components = 0;
    return DLP_OK;
  }
  if (num_inserted < 0 || num_edges < 0 || num_nodes <= 0 || !d_inserted_nodes || !d_component_id ||
      (num_edges > 0 && (!d_edge_src || !d_edge_dst)))
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "invalid arguments to dlp_connected_components");
  DLP_TRY(dlp::require_device());
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (num_edges == 0) {
    // src/connectedComponents.cu:191-205: ids left at -1, count = numInserted
    DLP_CUDA_TRY(cudaMemsetAsync(d_component_id, 0xff, sizeof(int) * static_cast<size_t>(num_nodes), s));
    *num_components = num_inserted;
    return DLP_OK;
  }
  const int words = (num_nodes + 31) / 32;
  const int chunks = (num_nodes + kChunkBits - 1) / kChunkBits;
  int *par = nullptr, *flags = nullptr, *err = nullptr, *chunk = nullptr, *total = nullptr;
  unsigned *bits = nullptr;
  dlp::GridBarrier *bar = nullptr;
  DLP_TRY(tmp_alloc(&par, num_nodes, s));
  DLP_TRY(tmp_alloc(&flags, kMaxHookRounds + 1, s));
  DLP_TRY(tmp_alloc(&err, 1, s));
  DLP_TRY(tmp_alloc(&bits, words, s));
  DLP_TRY(tmp_alloc(&chunk, chunks, s));
  DLP_TRY(tmp_alloc(&total, 1, s));
  DLP_TRY(tmp_alloc(&bar, 1, s));
  DLP_CUDA_TRY(cudaMemsetAsync(par, 0xff, sizeof(int) * static_cast<size_t>(num_nodes), s));
  DLP_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(int) * (kMaxHookRounds + 1), s));
  DLP_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  DLP_CUDA_TRY(cudaMemsetAsync(bits, 0, sizeof(unsigned) * words, s));
  DLP_CUDA_TRY(cudaMemsetAsync(bar, 0, sizeof(dlp::GridBarrier), s));
  cc_validate_init<<<grid_for(std::max(num_edges, num_inserted), kBlock), kBlock, 0, s>>>(
      d_edge_src, d_edge_dst, num_edges, d_inserted_nodes, num_inserted, num_nodes, par, err);
  DLP_CUDA_TRY(cudaGetLastError());
  CcArgs a{d_edge_src, d_edge_dst, num_edges, d_inserted_nodes, num_inserted, par, flags, bar, err,
           2000000000ull};
  const int grid = coop_grid(reinterpret_cast<const void *>(&cc_sv_kernel));
  if (grid <= 0) return dlp::fail(DLP_ERR_CUDA, "occupancy query failed");
  void *args[] = {&a};
  DLP_TRY(dlp::launch_cooperative(reinterpret_cast<const void *>(&cc_sv_kernel), grid, kBlock, args, 0, s));
  cc_mark_roots<<<grid_for(num_inserted, kBlock), kBlock, 0, s>>>(par, d_inserted_nodes, num_inserted, bits);
  cc_chunk_scan<<<1, 1024, 0, s>>>(bits, words, chunk, chunks, total);
  DLP_CUDA_TRY(cudaMemsetAsync(d_component_id, 0xff, sizeof(int) * static_cast<size_t>(num_nodes), s));
  cc_assign<<<grid_for(num_inserted, kBlock), kBlock, 0, s>>>(par, d_inserted_nodes, num_inserted, bits, chunk,
                                                             d_component_id);
  DLP_CUDA_TRY(cudaGetLastError());
  int host_err = 0, host_total = 0;
  DLP_CUDA_TRY(cudaMemcpyAsync(&host_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  DLP_CUDA_TRY(cudaMemcpyAsync(&host_total, total, sizeof(int), cudaMemcpyDeviceToHost, s));
  DLP_CUDA_TRY(cudaStreamSynchronize(s));
  for (void *p : {static_cast<void *>(par), static_cast<void *>(flags), static_cast<void *>(err),
                  static_cast<void *>(bits), static_cast<void *>(chunk), static_cast<void *>(total),
                  static_cast<void *>(bar)})
    cudaFreeAsync(p, s);
  if (host_err) return dlp::fail(host_err, "connected components failed on the device");
  *num_components = host_total;
  return DLP_OK;
}

int dlp_label_initialization(const int *d_row_ptr, const int *d_col_ind, const float *d_values, float *d_labels,
                             const int *d_vertex_status, const int *d_component_id, int num_components,
                             const int *d_inserted_nodes, int num_inserted, const int *d_gt_class, int num_nodes,
                             void *stream) {
  (void)d_vertex_status;  // not read by the reference either
  dlp::clear_error();
  if (num_inserted == 0) return DLP_OK;  // src/labelInitialization.cu:155
  if (num_inserted < 0 || num_nodes <= 0 || !d_row_ptr || !d_labels || !d_component_id || !d_inserted_nodes ||
      !d_gt_class)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "invalid arguments to dlp_label_initialization");
  DLP_TRY(dlp::require_device());
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nc = std::max(num_components, 1);
  long long *acc = nullptr;
  DLP_TRY(tmp_alloc(&acc, 2 * static_cast<size_t>(nc), s));
  DLP_CUDA_TRY(cudaMemsetAsync(acc, 0, sizeof(long long) * 2 * nc, s));
  init_accumulate<<<grid_for(static_cast<long long>(num_inserted) * kGroup, kBlock), kBlock, 0, s>>>(
      d_row_ptr, d_col_ind, d_values, d_component_id, num_components, d_gt_class, d_inserted_nodes, num_inserted,
      num_nodes, acc);
  init_labels<<<grid_for(num_inserted, kBlock), kBlock, 0, s>>>(d_labels, d_component_id, num_components, d_gt_class,
                                                               acc, d_inserted_nodes, num_inserted, num_nodes,
                                                               g_launcher_arith.load());
  DLP_CUDA_TRY(cudaGetLastError());
  DLP_CUDA_TRY(cudaFreeAsync(acc, s));
  return DLP_OK;
}

int dlp_iterative_propagation(const int *d_row_ptr, const int *d_col_ind, const float *d_values, float *d_labels,
                              float *d_labels_buffer, const int *d_vertex_status, const int *d_gt_class,
                              int *d_is_affected, int num_nodes, float delta, int max_iterations,
                              int *iterations_used, void *stream) {
  dlp::clear_error();
  if (!iterations_used) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null iterations_used");
  *iterations_used = 0;
  if (num_nodes <= 0 || !d_row_ptr || !d_labels || !d_labels_buffer || !d_vertex_status || !d_gt_class ||
      !d_is_affected)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "invalid arguments to dlp_iterative_propagation");
  DLP_TRY(dlp::require_device());
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = static_cast<size_t>(num_nodes);
  // both buffers start at the current labels (src/iterativePropagation.cu:268-270)
  DLP_CUDA_TRY(cudaMemcpyAsync(d_labels_buffer, d_labels, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
  unsigned *stamp = nullptr;
  int *lists = nullptr, *small = nullptr;
  dlp::GridBarrier *bar = nullptr;
  DLP_TRY(tmp_alloc(&stamp, n, s));
  DLP_TRY(tmp_alloc(&lists, 3 * n, s));
  DLP_TRY(tmp_alloc(&small, 16, s));
  DLP_TRY(tmp_alloc(&bar, 1, s));
  DLP_CUDA_TRY(cudaMemsetAsync(stamp, 0, sizeof(unsigned) * n, s));
  DLP_CUDA_TRY(cudaMemsetAsync(small, 0, sizeof(int) * 16, s));
  DLP_CUDA_TRY(cudaMemsetAsync(bar, 0, sizeof(dlp::GridBarrier), s));
  PropArgs a{};
  a.row_ptr = d_row_ptr;
  a.col = d_col_ind;
  a.val = d_values;
  a.labels = d_labels;
  a.buffer = d_labels_buffer;
  a.status = d_vertex_status;
  a.gt = d_gt_class;
  a.affected = d_is_affected;
  a.n = num_nodes;
  a.delta = delta;
  a.max_iter = max_iterations;
  a.stamp = stamp;
  a.lists = lists;
  a.counts = small;         // [0..5]
  a.out = small + 8;        // [8] passes
  a.err = small + 12;
  a.bar = bar;
  a.timeout_ns = 2000000000ull;
  a.fast_div = g_launcher_arith.load();
  const void *kern = prop_kernel_ptr(8);
  const int grid = coop_grid(kern);
  if (grid <= 0) return dlp::fail(DLP_ERR_CUDA, "occupancy query failed");
  void *args[] = {&a};
  DLP_TRY(dlp::launch_cooperative(kern, grid, kBlock, args, 0, s));
  int host[2] = {0, 0};
  DLP_CUDA_TRY(cudaMemcpyAsync(&host[0], a.out, sizeof(int), cudaMemcpyDeviceToHost, s));
  DLP_CUDA_TRY(cudaMemcpyAsync(&host[1], a.err, sizeof(int), cudaMemcpyDeviceToHost, s));
  DLP_CUDA_TRY(cudaStreamSynchronize(s));
  for (void *p : {static_cast<void *>(stamp), static_cast<void *>(lists), static_cast<void *>(small),
                  static_cast<void *>(bar)})
    cudaFreeAsync(p, s);
  if (host[1]) return dlp::fail(host[1], "propagation failed on the device");
  *iterations_used = host[0];
  return DLP_OK;
}

// dlp_iterative_propagation without any device allocation: the same kernel and
// results, with its scratch in g_noalloc_scratch instead of cudaMallocAsync
// temporaries. For callers that must not allocate device memory while they run
// (a framework that owns the whole device memory pool, a service that reserves
// its memory at start-up so nothing can fail or stall later). The first call
// on a device looks the array's address up; make that call before any stream
// capture. All calls share the one array, so calls that overlap on the GPU
// (other streams, other host threads) race; serialise them. Graphs of more
// than 2^20 vertices are rejected.
int dlp_iterative_propagation_noalloc(const int *d_row_ptr, const int *d_col_ind, const float *d_values,
                                      float *d_labels, float *d_labels_buffer, const int *d_vertex_status,
                                      const int *d_gt_class, int *d_is_affected, int num_nodes, float delta,
                                      int max_iterations, int *iterations_used, void *stream) {
  dlp::clear_error();
  if (!iterations_used) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null iterations_used");
  *iterations_used = 0;
  if (num_nodes <= 0 || !d_row_ptr || !d_labels || !d_labels_buffer || !d_vertex_status || !d_gt_class ||
      !d_is_affected)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "invalid arguments to dlp_iterative_propagation_noalloc");
  if (num_nodes > kNoAllocMaxNodes)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT,
                     "num_nodes " + std::to_string(num_nodes) + " exceeds the allocation-free limit of " +
                         std::to_string(kNoAllocMaxNodes) + " vertices; use dlp_iterative_propagation");
  DLP_TRY(dlp::require_device());
  NoAllocScratch *sc = nullptr;
  DLP_TRY(noalloc_scratch(&sc));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = static_cast<size_t>(num_nodes);
  DLP_CUDA_TRY(cudaMemcpyAsync(d_labels_buffer, d_labels, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
  // what must start at zero: the stamps in use, the counters, the barrier
  DLP_CUDA_TRY(cudaMemsetAsync(sc->stamp, 0, sizeof(unsigned) * n, s));
  DLP_CUDA_TRY(cudaMemsetAsync(sc->small, 0, sizeof(sc->small), s));
  DLP_CUDA_TRY(cudaMemsetAsync(&sc->bar, 0, sizeof(sc->bar), s));
  PropArgs a{};
  a.row_ptr = d_row_ptr;
  a.col = d_col_ind;
  a.val = d_values;
  a.labels = d_labels;
  a.buffer = d_labels_buffer;
  a.status = d_vertex_status;
  a.gt = d_gt_class;
  a.affected = d_is_affected;
  a.n = num_nodes;
  a.delta = delta;
  a.max_iter = max_iterations;
  a.stamp = sc->stamp;
  a.lists = sc->lists;
  a.counts = sc->small;
  a.out = sc->small + 8;
  a.err = sc->small + 12;
  a.bar = &sc->bar;
  a.timeout_ns = 2000000000ull;
  a.fast_div = g_launcher_arith.load();
  const void *kern = prop_kernel_ptr(8);
  const int grid = coop_grid(kern);
  if (grid <= 0) return dlp::fail(DLP_ERR_CUDA, "occupancy query failed");
  void *args[] = {&a};
  DLP_TRY(dlp::launch_cooperative(kern, grid, kBlock, args, 0, s));
  int host[2] = {0, 0};
  DLP_CUDA_TRY(cudaMemcpyAsync(&host[0], a.out, sizeof(int), cudaMemcpyDeviceToHost, s));
  DLP_CUDA_TRY(cudaMemcpyAsync(&host[1], a.err, sizeof(int), cudaMemcpyDeviceToHost, s));
  DLP_CUDA_TRY(cudaStreamSynchronize(s));
  if (host[1]) return dlp::fail(host[1], "propagation failed on the device");
  *iterations_used = host[0];
  return DLP_OK;
}

int dlp_irlp(const int *d_row_ptr, const int *d_col_ind, const float *d_values, float *d_labels,
             const int *d_vertex_status, const int *d_gt_class, int num_nodes, float delta, int max_iterations,
             int *iterations_used, void *stream) {
  dlp::clear_error();
  if (!iterations_used) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null iterations_used");
  *iterations_used = 0;
  if (num_nodes <= 0 || !d_row_ptr || !d_labels || !d_vertex_status || !d_gt_class)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "invalid arguments to dlp_irlp");
  DLP_TRY(dlp::require_device());
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = static_cast<size_t>(num_nodes);
  float *buffer = nullptr;
  int *small = nullptr;
  dlp::GridBarrier *bar = nullptr;
  DLP_TRY(tmp_alloc(&buffer, n, s));
  DLP_TRY(tmp_alloc(&small, 16, s));
  DLP_TRY(tmp_alloc(&bar, 1, s));
  DLP_CUDA_TRY(cudaMemcpyAsync(buffer, d_labels, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
  DLP_CUDA_TRY(cudaMemsetAsync(small, 0, sizeof(int) * 16, s));
  DLP_CUDA_TRY(cudaMemsetAsync(bar, 0, sizeof(dlp::GridBarrier), s));
  IrlpArgs a{d_row_ptr, d_col_ind, d_values, d_labels, buffer, d_vertex_status, d_gt_class, num_nodes, delta,
             max_iterations, small, bar, small + 8, 2000000000ull};
  const void *kern = reinterpret_cast<const void *>(&irlp_kernel);
  const int grid = coop_grid(kern);
  if (grid <= 0) return dlp::fail(DLP_ERR_CUDA, "occupancy query failed");
  void *args[] = {&a};
  DLP_TRY(dlp::launch_cooperative(kern, grid, kBlock, args, 0, s));
  int host[2] = {0, 0};
  DLP_CUDA_TRY(cudaMemcpyAsync(&host[0], small + 4, sizeof(int), cudaMemcpyDeviceToHost, s));
  DLP_CUDA_TRY(cudaMemcpyAsync(&host[1], small + 8, sizeof(int), cudaMemcpyDeviceToHost, s));
  DLP_CUDA_TRY(cudaStreamSynchronize(s));
  for (void *p : {static_cast<void *>(buffer), static_cast<void *>(small), static_cast<void *>(bar)})
    cudaFreeAsync(p, s);
  if (host[1]) return dlp::fail(host[1], "IrLP failed on the device");
  *iterations_used = host[0];
  return DLP_OK;
}

}  // extern "C"
