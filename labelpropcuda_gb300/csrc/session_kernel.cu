// The per-batch cooperative kernel of the resident session (see
// session_kernel.cuh for the phase map).
//
// Arithmetic that must agree bit for bit with the CPU oracle:
//   * a row's weighted average follows the reference's summation order: slot
//     t of a 256-slot block accumulates entries t, t+256, ... (add for the
//     weight, FMA for the weighted label) and the slots are folded by a tree
//     with strides 128..1 (src/iterativePropagation.cu:126-150). A row of at
//     most 32 entries only ever adds +0 at strides 128..32, so a group of G
//     lanes holding slots lane+G*r reproduces it exactly: in-register folds
//     for strides 16..G, then shuffles for G/2..1. Longer rows take a whole
//     warp holding slots lane+32*j (j = 0..7).
//   * the division is IEEE round-to-nearest (__fdiv_rn); the library is built
//     with -fmad=false so no other multiply-add is contracted.
//   * supernode weights are exact 32.32 fixed-point sums (order independent).
#include "session_kernel.cuh"

namespace dlp {
namespace session {
namespace {

struct Ctx {
  int gtid, nthreads, lane, gwarp, nwarps;
};

__device__ __forceinline__ Ctx make_ctx() {
  Ctx c;
  c.gtid = blockIdx.x * blockDim.x + threadIdx.x;
  c.nthreads = gridDim.x * blockDim.x;
  c.lane = threadIdx.x & 31;
  c.gwarp = c.gtid >> 5;
  c.nwarps = c.nthreads >> 5;
  return c;
}

__device__ __forceinline__ bool in_range(int v, int n) { return static_cast<unsigned>(v) < static_cast<unsigned>(n); }

struct View {
  const DevState &s;
  const BatchArgs &a;
  unsigned cur;   // this batch's stamp for del/gt/dirty marks
  unsigned g0;    // this batch's first frontier stamp

  __device__ bool inserted_now(int v) const {
    const int p = s.local[v];
    return p >= 0 && p < a.I && a.ins[p] == v;
  }
  // Same-batch deletion as the kernels see it (ref: the device status of a
  // vertex inserted and deleted in one batch is DELETED for that batch).
  __device__ bool dev_deleted(int v) const { return !a.spec && s.del_stamp[v] == cur; }
  // Live in the host rebuild of this batch (src/dynLP.cu:143-157).
  __device__ bool live(int v) const {
    if (s.status[v] == kDeleted) return false;
    if (s.batch_map) {
      const int m = s.batch_map[v];
      if (m < 0 || m > a.batch) return false;
    }
    return true;
  }
};

// Marks v affected with the batch's seed stamp; the first mark appends it to
// the raw seed list. Warp-convergent.
__device__ __forceinline__ void seed_mark(const View &w, bool cand, int v) {
  bool first = false;
  if (cand) first = atomicMax(&w.s.front_stamp[v], w.g0) < w.g0;
  warp_append(first, v, w.s.seed_list, &w.s.bc->num_seeds);
}

// Items [0, count) handled by groups of kRowGroup lanes; every lane of a warp
// runs the same number of chunk iterations so warp collectives stay legal.
template <class ItemFn>
__device__ __forceinline__ void grouped_rows(const Ctx &c, int count, ItemFn fn) {
  constexpr int GPW = 32 / kRowGroup;
  const int grp = c.lane / kRowGroup;
  const int gl = c.lane & (kRowGroup - 1);
  for (int base = c.gwarp * GPW; base < count; base += c.nwarps * GPW) {
    const int item = base + grp;
    fn(item, item < count, gl, grp);
  }
}

// ---------------------------------------------------------------- phase A ---
__device__ void phase_a(const View &w, const Ctx &c) {
  const DevState &s = w.s;
  const BatchArgs &a = w.a;
  const int n = s.n;
  int bad = 0;
  for (int i = c.gtid; i < a.I; i += c.nthreads) {
    const int v = a.ins[i];
    if (!in_range(v, n)) { bad = 1; continue; }
    s.local[v] = i;
    s.par[i] = i;
    s.acc[2 * i] = 0;
    s.acc[2 * i + 1] = 0;
    if (a.record) s.rec_minid[i] = 0x7fffffff;
  }
  for (int i = c.gtid; i < a.D; i += c.nthreads) {
    const int v = a.del[i];
    if (!in_range(v, n)) { bad = 1; continue; }
    if (a.spec) s.del_pre[i] = s.status[v];
    s.del_stamp[v] = w.cur;
  }
  for (int i = c.gtid; i < a.G; i += c.nthreads) {
    const int v = a.gt_ids[i];
    if (!in_range(v, n)) { bad = 1; continue; }
    s.gt_stamp[v] = w.cur;
  }
  for (int i = c.gtid; i < a.E; i += c.nthreads)
    if (!in_range(a.es[i], n) || !in_range(a.ed[i], n)) bad = 1;
  // Bring the stale label buffer back in line at the vertices the previous
  // batch's propagation wrote (both buffers start a batch equal,
  // src/dynLP.cu:519 and src/iterativePropagation.cu:268-270).
  if (a.seq > 0) {
    const int cb = s.ctl->cur_buf;
    const int tc = s.ctl->touched_count[(a.seq - 1) & 1];
    const int *list = s.touched + static_cast<size_t>((a.seq - 1) & 1) * n;
    float *dst = cb ? s.lab0 : s.lab1;
    const float *src = cb ? s.lab1 : s.lab0;
    for (int i = c.gtid; i < tc; i += c.nthreads) {
      const int v = list[i];
      dst[v] = src[v];
    }
  }
  if (c.gtid == 0) s.ctl->touched_count[a.seq & 1] = 0;
  if (bad) atomicCAS(&s.ctl->err, 0, DLP_ERR_INVALID_ARGUMENT);
}

// ---------------------------------------------------------------- phase B ---
// Host-status update (ref: delete, insert, then ground truth,
// src/dynLP.cu:117-130; spec: deletions win) and dirty-row marking.
__device__ void phase_b(const View &w, const Ctx &c) {
  const DevState &s = w.s;
  const BatchArgs &a = w.a;
  for (int i = c.gtid; i < a.D; i += c.nthreads) {
    const int v = a.del[i];
    if (a.spec || (!w.inserted_now(v) && s.gt_stamp[v] != w.cur)) s.status[v] = kDeleted;
  }
  for (int i = c.gtid; i < a.I; i += c.nthreads) {
    const int v = a.ins[i];
    if (s.gt_stamp[v] == w.cur) continue;
    if (a.spec && s.del_stamp[v] == w.cur) continue;
    s.status[v] = kActive;
  }
  for (int i = c.gtid; i < a.G; i += c.nthreads) {
    const int v = a.gt_ids[i];
    const float l = a.gt_lab[i];
    s.gt[v] = l < 0.5f ? 0 : 1;
    s.lab0[v] = l;
    s.lab1[v] = l;
    if (!(a.spec && s.del_stamp[v] == w.cur)) s.status[v] = kGroundTruth;
  }
  // Rows whose live content can change: every changed vertex and its
  // full-graph neighbours. The previous batch's deletions are included so
  // that a same-batch insert+delete (ref) gets its row back.
  const int total = a.D + a.I + a.PD + a.G;
  grouped_rows(c, total, [&](int item, bool valid, int gl, int) {
    int x = -1;
    if (valid) {
      int k = item;
      if (k < a.D) x = a.del[k];
      else if ((k -= a.D) < a.I) x = a.ins[k];
      else if ((k -= a.I) < a.PD) x = a.prev_del[k];
      else x = a.gt_ids[k - a.PD];
    }
    const int rs = valid ? s.full_row[x] : 0;
    const int len = valid ? s.full_row[x + 1] - rs : 0;
    const int maxlen = __reduce_max_sync(0xffffffffu, len + 1);  // +1: the vertex itself
    for (int off = 0; off < maxlen; off += kRowGroup) {
      const int e = off + gl - 1;  // e == -1: x itself
      int v = -1;
      if (valid && e < len) v = e < 0 ? x : s.full_adj[rs + e].x;
      bool first = false;
      if (v >= 0) first = atomicMax(&s.dirty_stamp[v], w.cur) < w.cur;
      warp_append(first, v, s.dirty_list, &s.bc->num_dirty);
    }
  });
}

// ---------------------------------------------------------------- phase C ---
// Live-row compaction of dirty rows, deletion marks and the tau filter.
__device__ void phase_c(const View &w, const Ctx &c) {
  const DevState &s = w.s;
  const BatchArgs &a = w.a;
  const int ndirty = s.bc->num_dirty;
  grouped_rows(c, ndirty, [&](int item, bool valid, int gl, int grp) {
    int u = 0, rs = 0, len = 0;
    bool keep_row = false, del_row = false;
    if (valid) {
      u = s.dirty_list[item];
      keep_row = w.live(u);
      rs = s.full_row[u];
      len = keep_row ? s.full_row[u + 1] - rs : 0;
      del_row = keep_row && w.dev_deleted(u);
    }
    const int maxlen = __reduce_max_sync(0xffffffffu, len);
    const int entries = __reduce_add_sync(0xffffffffu, gl == 0 ? len : 0);
    if (c.lane == 0 && entries) atomicAdd(&s.bc->dirty_entries, static_cast<unsigned long long>(entries));
    const unsigned gmask = ((1u << kRowGroup) - 1u) << (grp * kRowGroup);
    int pos = 0;
    for (int off = 0; off < maxlen; off += kRowGroup) {
      const int e = off + gl;
      bool keep = false;
      int2 ent = make_int2(-1, 0);
      if (e < len) {
        ent = s.full_adj[rs + e];
        keep = ent.x >= 0 && w.live(ent.x);
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep) & gmask;
      if (keep) {
        const int rank = __popc(m & ((1u << c.lane) - 1u));
        int col = ent.x;
        // Soft delete (src/sparsifySubgraph.cu:78,108): entries of a row that
        // is deleted this batch, and entries pointing at such a vertex.
        if (del_row || w.dev_deleted(col)) col = -1;
        s.act_adj[rs + pos + rank] = make_int2(col, ent.y);
      }
      // Neighbours of a deleted vertex's live row are affected
      // (src/sparsifySubgraph.cu:71-76; empty unless inserted this batch).
      seed_mark(w, keep && del_row, ent.x);
      pos += __popc(m);
    }
    if (valid && gl == 0) s.act_len[u] = keep_row ? pos : 0;
  });

  if (a.spec) {
    // spec: neighbours of every deleted vertex that was live before this
    // batch's deletions, in the adjacency before the deletion
    grouped_rows(c, a.D, [&](int item, bool valid, int gl, int) {
      int x = 0;
      bool was = false;
      if (valid) {
        x = a.del[item];
        was = s.del_pre[item] != kDeleted || w.inserted_now(x) || s.gt_stamp[x] == w.cur;
        if (was && s.batch_map) {
          const int m = s.batch_map[x];
          was = m >= 0 && m <= a.batch;
        }
      }
      const int rs = was ? s.full_row[x] : 0;
      const int len = was ? s.full_row[x + 1] - rs : 0;
      const int maxlen = __reduce_max_sync(0xffffffffu, len);
      for (int off = 0; off < maxlen; off += kRowGroup) {
        const int e = off + gl;
        const int v = e < len ? s.full_adj[rs + e].x : -1;
        seed_mark(w, v >= 0 && w.live(v), v);
      }
    });
  }

  // Tau filter over the batch's raw edges: local endpoints for the components
  // step, kept new-new edges, and endpoint marks.
  const bool comp_path = a.spec ? (a.I > 0) : (a.I > 0 && a.E > 0);
  if (!comp_path) return;
  const bool vec = ((reinterpret_cast<uintptr_t>(a.es) | reinterpret_cast<uintptr_t>(a.ed) |
                     reinterpret_cast<uintptr_t>(a.ew) | reinterpret_cast<uintptr_t>(s.lsrc) |
                     reinterpret_cast<uintptr_t>(s.ldst)) & 15u) == 0;
  const int nvec = vec ? (a.E >> 2) : 0;
  auto one_edge = [&](bool valid, int sv, int dv, float wt, int &ls, int &ld) {
    ls = -1;
    ld = -1;
    bool kept = false;
    if (valid) {
      ls = w.inserted_now(sv) ? s.local[sv] : -1;
      ld = w.inserted_now(dv) ? s.local[dv] : -1;
      kept = wt > a.tau && ls >= 0 && ld >= 0;
    }
    // kept new-new edge (src/sparsifySubgraph.cu:133,165-174), written as
    // (src,dst) and its inserted positions
    const unsigned m = __ballot_sync(0xffffffffu, kept);
    if (m) {
      const int leader = __ffs(m) - 1;
      int base = 0;
      if (c.lane == leader) base = atomicAdd(&s.bc->num_kept, __popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (kept) {
        const int k = base + __popc(m & ((1u << c.lane) - 1u));
        s.sub_pairs[2 * k] = sv;
        s.sub_pairs[2 * k + 1] = dv;
        s.sub_local[2 * k] = ls;
        s.sub_local[2 * k + 1] = ld;
      }
    }
    if (!a.spec) {
      // ref: endpoints of edges with w > tau, clipped to ids below the
      // inserted count (src/sparsifySubgraph.cu:259-263 with :177-178)
      const bool heavy = valid && wt > a.tau;
      seed_mark(w, heavy && sv < a.I, sv);
      seed_mark(w, heavy && dv < a.I, dv);
    } else {
      seed_mark(w, valid && w.live(sv), sv);
      seed_mark(w, valid && w.live(dv), dv);
    }
  };
  // int4/float4 body: four edges per lane
  for (int base = c.gwarp * 32; base < nvec; base += c.nwarps * 32) {
    const int q = base + c.lane;
    const bool valid = q < nvec;
    int4 s4 = make_int4(0, 0, 0, 0), d4 = s4;
    float4 w4 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) {
      s4 = reinterpret_cast<const int4 *>(a.es)[q];
      d4 = reinterpret_cast<const int4 *>(a.ed)[q];
      w4 = reinterpret_cast<const float4 *>(a.ew)[q];
    }
    int4 l4, m4;
    one_edge(valid, s4.x, d4.x, w4.x, l4.x, m4.x);
    one_edge(valid, s4.y, d4.y, w4.y, l4.y, m4.y);
    one_edge(valid, s4.z, d4.z, w4.z, l4.z, m4.z);
    one_edge(valid, s4.w, d4.w, w4.w, l4.w, m4.w);
    if (valid) {
      reinterpret_cast<int4 *>(s.lsrc)[q] = l4;
      reinterpret_cast<int4 *>(s.ldst)[q] = m4;
    }
  }
  // scalar tail (or everything when the arrays are not 16-byte aligned)
  const int first = nvec * 4;
  for (int base = first + c.gwarp * 32; base < a.E; base += c.nwarps * 32) {
    const int i = base + c.lane;
    const bool valid = i < a.E;
    int ls, ld;
    one_edge(valid, valid ? a.es[i] : 0, valid ? a.ed[i] : 0, valid ? a.ew[i] : 0.f, ls, ld);
    if (valid) {
      s.lsrc[i] = ls;
      s.ldst[i] = ld;
    }
  }
  if (a.spec) {
    // spec: every new non-ground-truth vertex is affected
    for (int base = c.gwarp * 32; base < a.I; base += c.nwarps * 32) {
      const int i = base + c.lane;
      const int v = i < a.I ? a.ins[i] : 0;
      seed_mark(w, i < a.I && s.gt[v] < 0 && w.live(v), v);
    }
  }
}

// Appends v to the frontier set `set` (narrow list from the front, wide from
// the back) and, the first time this batch, to the touched list.
__device__ __forceinline__ void frontier_append(const View &w, bool pred, bool first, int v,
                                                int set) {
  const DevState &s = w.s;
  bool wide = false;
  if (pred) wide = s.act_len[v] > kNarrowMax;
  int *list = s.flist + static_cast<size_t>(set) * s.n;
  warp_append(pred && !wide, v, list, &s.bc->front_count[set][0]);
  warp_append_back(pred && wide, v, list, s.n, &s.bc->front_count[set][1]);
  warp_append(first, v, s.touched + static_cast<size_t>(w.a.seq & 1) * s.n,
              &s.ctl->touched_count[w.a.seq & 1]);
}

// ---------------------------------------------------------------- phase D ---
__device__ void phase_d_frontier(const View &w, const Ctx &c) {
  const DevState &s = w.s;
  const int ns = s.bc->num_seeds;
  for (int base = c.gwarp * 32; base < ns; base += c.nwarps * 32) {
    const int i = base + c.lane;
    int v = 0;
    bool ok = false;
    if (i < ns) {
      v = s.seed_list[i];
      // collect filter (src/iterativePropagation.cu:73-75)
      ok = s.status[v] == kActive && !w.dev_deleted(v) && s.gt[v] < 0;
    }
    frontier_append(w, ok, ok, v, 0);
    if (w.a.record) warp_append(ok, v, s.rec_front0, &s.bc->seed_frontier);
    else {
      const unsigned m = __ballot_sync(0xffffffffu, ok);
      if (c.lane == 0 && m) atomicAdd(&s.bc->seed_frontier, __popc(m));
    }
  }
}

// One hook pass: roots of each edge's endpoints, larger root hooked under the
// smaller with atomicMin (src/connectedComponents.cu:79-100). Inserted
// positions are the node ids; -1 stands for a vertex that is not new in this
// batch (the reference's par == -1 entries).
__device__ void sv_hook(const View &w, const Ctx &c, const int *A, const int *B, int stride,
                        int count, int round) {
  const DevState &s = w.s;
  bool changed = false;
  for (int i = c.gtid; i < count; i += c.nthreads) {
    const int x = A[static_cast<size_t>(i) * stride];
    const int y = B[static_cast<size_t>(i) * stride];
    const int rx = x < 0 ? -1 : s.par[x];
    const int ry = y < 0 ? -1 : s.par[y];
    if (rx != ry) {
      const int hi = max(rx, ry), lo = min(rx, ry);
      if (atomicMin(&s.par[hi], lo) != lo) changed = true;
    }
  }
  if (__any_sync(0xffffffffu, changed) && c.lane == 0) s.bc->hook_flag[round] = 1;
}

// Pointer jumping to the root in one pass (the reference repeats
// par[v] = par[par[v]] until nothing changes, src/connectedComponents.cu:108-121,
// which ends in the same state). Chains strictly decrease, so the walk ends.
__device__ void sv_compress(const View &w, const Ctx &c) {
  const DevState &s = w.s;
  for (int i = c.gtid; i < w.a.I; i += c.nthreads) {
    int p = s.par[i];
    while (p >= 0) {
      const int q = s.par[p];
      if (q == p) break;
      p = q;
    }
    s.par[i] = p;
  }
}

// ---------------------------------------------------------------- phase E ---
// Component count and fixed-point supernode weights per component root
// (src/labelInitialization.cu:59-88).
__device__ void phase_e(const View &w, const Ctx &c) {
  const DevState &s = w.s;
  const BatchArgs &a = w.a;
  int roots = 0;
  for (int i = c.gtid; i < a.I; i += c.nthreads) {
    const int p = s.par[i];
    if (p == i) ++roots;
    if (a.record && p >= 0) atomicMin(&s.rec_minid[p], a.ins[i]);
  }
  roots = warp_sum_i(roots);
  if (c.lane == 0 && roots) atomicAdd(&s.bc->num_comp, roots);

  grouped_rows(c, a.I, [&](int item, bool valid, int gl, int) {
    int rs = 0, len = 0, root = -1;
    if (valid) {
      root = s.par[item];
      const int u = a.ins[item];
      if (root >= 0) {
        rs = s.full_row[u];
        len = s.act_len[u];
      }
    }
    const int maxlen = __reduce_max_sync(0xffffffffu, len);
    long long q0 = 0, q1 = 0;
    for (int off = 0; off < maxlen; off += kRowGroup) {
      const int e = off + gl;
      if (e < len) {
        const int2 ent = s.act_adj[rs + e];
        if (ent.x >= 0) {
          const int g = s.gt[ent.x];
          const long long q = to_fixed(__int_as_float(ent.y));
          if (g == 0) q0 += q;
          else if (g == 1) q1 += q;
        }
      }
    }
#pragma unroll
    for (int o = kRowGroup / 2; o > 0; o >>= 1) {
      q0 += __shfl_down_sync(0xffffffffu, q0, o, kRowGroup);
      q1 += __shfl_down_sync(0xffffffffu, q1, o, kRowGroup);
    }
    if (valid && gl == 0 && root >= 0) {
      if (q0) atomicAdd(reinterpret_cast<unsigned long long *>(&s.acc[2 * root]),
                        static_cast<unsigned long long>(q0));
      if (q1) atomicAdd(reinterpret_cast<unsigned long long *>(&s.acc[2 * root + 1]),
                        static_cast<unsigned long long>(q1));
    }
  });
}

// ---------------------------------------------------------------- phase F ---
__device__ void phase_f(const View &w, const Ctx &c, bool comp_path) {
  const DevState &s = w.s;
  const BatchArgs &a = w.a;
  for (int i = c.gtid; i < a.I; i += c.nthreads) {
    const int u = a.ins[i];
    float l;
    if (comp_path) {
      // src/labelInitialization.cu:99-142
      const int g = s.gt[u];
      const int root = s.par[i];
      if (g == 0) l = 0.0f;
      else if (g == 1) l = 1.0f;
      else if (root < 0) l = 0.5f;
      else {
        const float w0 = from_fixed(s.acc[2 * root]);
        const float w1 = from_fixed(s.acc[2 * root + 1]);
        const float den = w0 + w1;
        l = den > 1e-10f ? __fdiv_rn(w1, den) : 0.5f;
      }
      s.lab0[u] = l;
      s.lab1[u] = l;
    } else {
      // new vertices without new edges (src/dynLP.cu:482-504): this batch's
      // ground truth keeps the label set in phase B, everything else 0.5
      if (s.gt_stamp[u] == w.cur && s.gt[u] >= 0) {
        l = s.lab0[u];
      } else {
        l = 0.5f;
        s.lab0[u] = l;
        s.lab1[u] = l;
      }
    }
    if (a.record) {
      s.rec_init[i] = l;
      const int root = comp_path ? s.par[i] : i;
      s.rec_root[i] = (!comp_path || root < 0) ? -1 : s.rec_minid[root];
    }
  }
}

// ---------------------------------------------------------------- phase G ---
// Frontier propagation until the frontier is empty (src/iterativePropagation.cu:274-327).

// One row of at most 32 live entries by a group of G lanes: new label into
// dst, then mark(cand, v) for each entry and for u itself (called by every
// lane, the same number of times). Returns whether u moved by more than delta.
template <int G, class Mark>
__device__ __forceinline__ void narrow_row(const DevState &s, const float *src, float *dst, float delta, int u,
                                           bool valid, int gl, unsigned long long &edges,
                                           unsigned long long &visits, Mark mark) {
  constexpr int R = 32 / G;
  int rs = 0, len = 0;
  if (valid) {
    rs = s.full_row[u];
    len = s.act_len[u];
  }
  float sw[R], sl[R];
  int vv[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int e = gl + G * r;
    sw[r] = 0.0f;
    sl[r] = 0.0f;
    vv[r] = -1;
    if (e < len) {
      const int2 ent = s.act_adj[rs + e];
      vv[r] = ent.x;
      if (ent.x >= 0) {
        const float wt = __int_as_float(ent.y);
        sw[r] = wt;                                // 0 + w
        sl[r] = __fmaf_rn(wt, src[ent.x], 0.0f);   // fma(w, F_v, 0)
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
  int changed = 0;
  if (valid && gl == 0) {
    const float old = src[u];
    const float nl = updated_label(tw, tl, old);
    dst[u] = nl;
    changed = fabsf(nl - old) > delta;
    edges += static_cast<unsigned long long>(len);
    visits += 1ull;
  }
  changed = __shfl_sync(0xffffffffu, changed, 0, G);
  // changed vertex: non-deleted, non-GT neighbours and itself
  // (src/iterativePropagation.cu:200-216)
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int v = vv[r];
    mark(changed && v >= 0 && s.gt[v] < 0, v);
  }
  mark(changed && gl == 0, u);
}

// One row of any length by a whole warp: 256 slots held as lane + 32*j.
template <class Mark>
__device__ __forceinline__ void wide_row(const DevState &s, const float *src, float *dst, float delta, int u,
                                         int lane, unsigned long long &edges, unsigned long long &visits,
                                         Mark mark) {
  const int rs = s.full_row[u];
  const int len = s.act_len[u];
  float sw[8], sl[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) sw[j] = sl[j] = 0.0f;
  for (int p = 0; p < len; p += 256) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int e = p + j * 32 + lane;
      if (e < len) {
        const int2 ent = s.act_adj[rs + e];
        if (ent.x >= 0) {
          const float wt = __int_as_float(ent.y);
          sw[j] = sw[j] + wt;
          sl[j] = __fmaf_rn(wt, src[ent.x], sl[j]);
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
  int changed = 0;
  if (lane == 0) {
    const float old = src[u];
    const float nl = updated_label(tw, tl, old);
    dst[u] = nl;
    changed = fabsf(nl - old) > delta;
    edges += static_cast<unsigned long long>(len);
    visits += 1ull;
  }
  changed = __shfl_sync(0xffffffffu, changed, 0);
  if (changed) {
    for (int e0 = 0; e0 < len; e0 += 32) {
      const int e = e0 + lane;
      const int v = e < len ? s.act_adj[rs + e].x : -1;
      mark(v >= 0 && s.gt[v] < 0, v);
    }
    mark(lane == 0, u);
  }
}

// Solo mode: small frontiers are run by block 0 alone, pass after pass, with
// __syncthreads() between passes and the frontier and its dedup set in shared
// memory, while the other blocks wait at the next grid barrier. The passes and
// their arithmetic are exactly those of the grid path; only the
// synchronisation changes. Solo mode ends at the first pass whose frontier is
// too large for the shared buffers, when the frontier empties, at max_iter,
// or after kSoloBudgetNs, and hands the frontier back through the global set.
constexpr int kSoloEntry = 128;       // enter when the frontier is at most this
constexpr int kSoloLive = 512;        // leave when it grows above this
constexpr int kSoloCap = 1024;        // shared frontier capacity (next pass bound)
constexpr int kSoloHash = 2048;       // per-pass dedup table
constexpr int kSoloSeen = 2048;       // vertices that entered a frontier in solo mode
constexpr unsigned long long kSoloBudgetNs = 100000000ull;

struct SoloShared {
  int list[2][kSoloCap];
  int hash[kSoloHash];
  int seen[kSoloSeen];
  int cnt[2][2];
  int seen_n;
  int stop;
  int bound;
};

__device__ __forceinline__ unsigned mix32(unsigned x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// Inserts v into an open-addressing table of `size` slots (-1 = empty);
// returns true when v was not present. The caller bounds the load.
__device__ __forceinline__ bool shared_insert(int *table, int size, int v) {
  unsigned h = mix32(static_cast<unsigned>(v)) & static_cast<unsigned>(size - 1);
  for (int probe = 0; probe < size; ++probe) {
    const int prev = atomicCAS(&table[h], -1, v);
    if (prev == -1) return true;
    if (prev == v) return false;
    h = (h + 1) & static_cast<unsigned>(size - 1);
  }
  return false;
}

template <int G>
__device__ int solo_passes(const View &w, int k0, SoloShared &sh, unsigned long long &edges,
                           unsigned long long &visits) {
  const DevState &s = w.s;
  const BatchArgs &a = w.a;
  const int n = s.n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int GPW = 32 / G;
  const int grp = lane / G, gl = lane & (G - 1);
  const int cb = s.ctl->cur_buf;
  // take over F_k0 from the global set
  {
    const int set = k0 % 3;
    const int nn = ld_relaxed_i32(&s.bc->front_count[set][0]);
    const int nw = ld_relaxed_i32(&s.bc->front_count[set][1]);
    const int *gl_list = s.flist + static_cast<size_t>(set) * n;
    for (int i = tid; i < nn; i += blockDim.x) sh.list[0][i] = gl_list[i];
    for (int i = tid; i < nw; i += blockDim.x) sh.list[0][kSoloCap - 1 - i] = gl_list[n - 1 - i];
    for (int i = tid; i < kSoloSeen; i += blockDim.x) sh.seen[i] = -1;
    if (tid == 0) {
      sh.cnt[0][0] = nn;
      sh.cnt[0][1] = nw;
      sh.seen_n = 0;
    }
  }
  __syncthreads();
  const uint64_t t0 = global_timer_ns();
  int k = k0;
  int p = 0;
  for (;; ++k, p ^= 1) {
    const int nn = sh.cnt[p][0], nw = sh.cnt[p][1];
    // next-frontier bound: every live entry of every frontier row, plus the rows
    if (tid == 0) sh.bound = nn + nw;
    __syncthreads();
    int part = 0;
    for (int i = tid; i < nn; i += blockDim.x) part += s.act_len[sh.list[p][i]];
    for (int i = tid; i < nw; i += blockDim.x) part += s.act_len[sh.list[p][kSoloCap - 1 - i]];
    part = warp_sum_i(part);
    if (lane == 0 && part) atomicAdd(&sh.bound, part);
    if (tid == 0) {
      int stop = 0;
      if (nn + nw == 0 || k >= a.max_iter || nn + nw > kSoloLive) stop = 1;
      if (sh.bound > kSoloCap || sh.seen_n + sh.bound > kSoloSeen / 2) stop = 1;
      if (((k - k0) & 31) == 31 && global_timer_ns() - t0 > kSoloBudgetNs) stop = 1;
      sh.stop = stop;
    }
    for (int i = tid; i < kSoloHash; i += blockDim.x) sh.hash[i] = -1;
    if (tid == 0) {
      sh.cnt[p ^ 1][0] = 0;
      sh.cnt[p ^ 1][1] = 0;
    }
    __syncthreads();
    if (sh.stop) break;
    if (tid == 0 && a.record && k < kRecordIters) s.rec_fsizes[k] = nn + nw;
    const float *src = ((cb ^ k) & 1) ? s.lab1 : s.lab0;
    float *dst = ((cb ^ k) & 1) ? s.lab0 : s.lab1;
    int *next = sh.list[p ^ 1];
    auto mark = [&](bool cand, int v) {
      if (!cand || !shared_insert(sh.hash, kSoloHash, v)) return;
      if (s.act_len[v] > kNarrowMax) next[kSoloCap - 1 - atomicAdd(&sh.cnt[p ^ 1][1], 1)] = v;
      else next[atomicAdd(&sh.cnt[p ^ 1][0], 1)] = v;
      if (shared_insert(sh.seen, kSoloSeen, v)) atomicAdd(&sh.seen_n, 1);
    };
    for (int base = warp * GPW; base < nn; base += (blockDim.x >> 5) * GPW) {
      const int item = base + grp;
      const bool valid = item < nn;
      narrow_row<G>(s, src, dst, a.delta, valid ? sh.list[p][item] : 0, valid, gl, edges, visits, mark);
    }
    for (int wi = warp; wi < nw; wi += blockDim.x >> 5)
      wide_row(s, src, dst, a.delta, sh.list[p][kSoloCap - 1 - wi], lane, edges, visits, mark);
    __syncthreads();
  }
  // hand F_k back to the grid: global set k%3, empty set (k+1)%3
  {
    const int set = k % 3;
    const int nn = sh.cnt[p][0], nw = sh.cnt[p][1];
    int *gl_list = s.flist + static_cast<size_t>(set) * n;
    for (int i = tid; i < nn; i += blockDim.x) gl_list[i] = sh.list[p][i];
    for (int i = tid; i < nw; i += blockDim.x) gl_list[n - 1 - i] = sh.list[p][kSoloCap - 1 - i];
    if (tid == 0) {
      s.bc->front_count[set][0] = nn;
      s.bc->front_count[set][1] = nw;
      s.bc->front_count[(k + 1) % 3][0] = 0;
      s.bc->front_count[(k + 1) % 3][1] = 0;
      s.bc->solo_k = k;
      s.bc->solo_passes = k - k0;
    }
    // vertices that first entered a frontier in solo mode join the touched
    // list; their stamps stay below the next grid pass's stamp
    const unsigned st = w.g0 + static_cast<unsigned>(k);
    int *tl = s.touched + static_cast<size_t>(a.seq & 1) * n;
    for (int i = tid; i < kSoloSeen; i += blockDim.x) {
      const int v = sh.seen[i];
      if (v < 0) continue;
      const unsigned old = atomicMax(&s.front_stamp[v], st);
      if (old < w.g0) tl[atomicAdd(&s.ctl->touched_count[a.seq & 1], 1)] = v;
    }
  }
  return k;
}

template <int G>
__device__ bool phase_g(const View &w, const Ctx &c, int &iterations, unsigned long long &edges,
                        unsigned long long &visits, SoloShared &solo) {
  const DevState &s = w.s;
  const BatchArgs &a = w.a;
  const int n = s.n;
  constexpr int GPW = 32 / G;
  const int grp = c.lane / G;
  const int gl = c.lane & (G - 1);
  const int cb = s.ctl->cur_buf;
  int k = 0;
  int no_solo_at = -1;  // a pass solo mode declined to run goes to the grid
  for (;; ++k) {
    const int set = k % 3;
    const int nn = ld_relaxed_i32(&s.bc->front_count[set][0]);
    const int nw = ld_relaxed_i32(&s.bc->front_count[set][1]);
    if (nn + nw == 0 || k >= a.max_iter) break;
    if (a.solo && nn + nw <= kSoloEntry && k != no_solo_at) {
      if (blockIdx.x == 0) solo_passes<G>(w, k, solo, edges, visits);
      if (!grid_sync(&s.ctl->bar, &s.ctl->err, a.timeout_ns)) return false;
      const int done = ld_relaxed_i32(&s.bc->solo_passes);
      const int kk = ld_relaxed_i32(&s.bc->solo_k);
      if (done == 0) no_solo_at = k;
      k = kk - 1;  // the loop increment resumes at pass kk
      continue;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      // the set filled two passes from now was last read one pass ago
      s.bc->front_count[(k + 2) % 3][0] = 0;
      s.bc->front_count[(k + 2) % 3][1] = 0;
      if (a.record && k < kRecordIters) s.rec_fsizes[k] = nn + nw;
    }
    const float *src = ((cb ^ k) & 1) ? s.lab1 : s.lab0;
    float *dst = ((cb ^ k) & 1) ? s.lab0 : s.lab1;
    const unsigned stamp = w.g0 + static_cast<unsigned>(k) + 1u;
    const int nset = (k + 1) % 3;
    const int *cur_list = s.flist + static_cast<size_t>(set) * n;
    auto mark = [&](bool cand, int v) {
      bool fresh = false, first = false;
      if (cand) {
        const unsigned old = atomicMax(&s.front_stamp[v], stamp);
        fresh = old < stamp;
        first = old < w.g0;
      }
      frontier_append(w, fresh, first, v, nset);
    };
    for (int base = c.gwarp * GPW; base < nn; base += c.nwarps * GPW) {
      const int item = base + grp;
      const bool valid = item < nn;
      narrow_row<G>(s, src, dst, a.delta, valid ? cur_list[item] : 0, valid, gl, edges, visits, mark);
    }
    for (int wi = c.gwarp; wi < nw; wi += c.nwarps)
      wide_row(s, src, dst, a.delta, cur_list[n - 1 - wi], c.lane, edges, visits, mark);
    if (!grid_sync(&s.ctl->bar, &s.ctl->err, a.timeout_ns)) return false;
  }
  iterations = k;
  return true;
}

// ---------------------------------------------------------------- phase H ---
__device__ void phase_h(const View &w, const Ctx &c, int new_buf) {
  const DevState &s = w.s;
  const BatchArgs &a = w.a;
  // ground truth of this batch back to exactly 0 / 1 in both buffers
  // (src/iterativePropagation.cu:224-235; earlier ground truth already is)
  for (int i = c.gtid; i < a.G; i += c.nthreads) {
    const int v = a.gt_ids[i];
    const float l = s.gt[v] == 0 ? 0.0f : 1.0f;
    s.lab0[v] = l;
    s.lab1[v] = l;
  }
  // accuracy (src/dynLP.cu:65-85), updated at every vertex whose status or
  // label may have changed
  const float *lab = new_buf ? s.lab1 : s.lab0;
  const int tc = s.ctl->touched_count[a.seq & 1];
  const int *tl = s.touched + static_cast<size_t>(a.seq & 1) * s.n;
  const int total = tc + a.I + a.D + a.G;
  long long dc = 0, dt = 0;
  for (int k = c.gtid; k < total; k += c.nthreads) {
    int i = k, v;
    if (i < tc) v = tl[i];
    else if ((i -= tc) < a.I) v = a.ins[i];
    else if ((i -= a.I) < a.D) v = a.del[i];
    else v = a.gt_ids[i - a.D];
    const int st = s.status[v];
    int now = -1;
    if (st != kDeleted && st != kGroundTruth) {
      const int pred = lab[v] >= 0.5f ? 1 : 0;
      const int truth = s.truth ? s.truth[v] : 0;
      now = pred == truth ? 1 : 0;
    }
    const int before = atomicExch(&s.contrib[v], now);
    dc += (now == 1) - (before == 1);
    dt += (now >= 0) - (before >= 0);
  }
  dc = warp_sum_ll(dc);
  dt = warp_sum_ll(dt);
  if (c.lane == 0 && (dc || dt)) {
    atomicAdd(reinterpret_cast<unsigned long long *>(&s.ctl->correct), static_cast<unsigned long long>(dc));
    atomicAdd(reinterpret_cast<unsigned long long *>(&s.ctl->total), static_cast<unsigned long long>(dt));
  }
}

}  // namespace

template <int G>
__global__ void __launch_bounds__(kBlock) batch_kernel(DevState s, BatchArgs a) {
  const Ctx c = make_ctx();
  const unsigned base = s.ctl->stamp_base;
  const View w{s, a, static_cast<unsigned>(a.seq) + 1u, base + 1u};
  const uint64_t to = a.timeout_ns;
  GridBarrier *bar = &s.ctl->bar;
  int *err = &s.ctl->err;
  if (ld_relaxed_i32(err) != 0) return;

  phase_a(w, c);
  if (!grid_sync(bar, err, to)) return;
  phase_b(w, c);
  if (!grid_sync(bar, err, to)) return;
  phase_c(w, c);
  if (!grid_sync(bar, err, to)) return;

  const bool comp_path = a.spec ? (a.I > 0) : (a.I > 0 && a.E > 0);
  phase_d_frontier(w, c);
  int hook_count = 0;
  const int *ha = nullptr, *hb = nullptr;
  int hstride = 1;
  if (comp_path) {
    const int kept = s.bc->num_kept;
    if (a.spec) {
      hook_count = kept;
      ha = s.sub_local;
      hb = s.sub_local + 1;
      hstride = 2;
    } else if (kept > 0) {
      // the reference hooks the first numSubEdges RAW edges (src/dynLP.cu:437-440)
      hook_count = min(2 * kept, a.E);
      ha = s.lsrc;
      hb = s.ldst;
    }
  }
  int rounds = 0;
  if (hook_count > 0) {
    for (int r = 0; r < kMaxHookRounds; ++r) {
      sv_hook(w, c, ha, hb, hstride, hook_count, r);
      if (!grid_sync(bar, err, to)) return;
      sv_compress(w, c);
      if (!grid_sync(bar, err, to)) return;
      rounds = r + 1;
      if (ld_relaxed_i32(&s.bc->hook_flag[r]) == 0) break;
    }
  } else {
    if (!grid_sync(bar, err, to)) return;
  }

  if (comp_path) {
    phase_e(w, c);
    if (!grid_sync(bar, err, to)) return;
  }
  phase_f(w, c, comp_path);
  if (!grid_sync(bar, err, to)) return;

  int iterations = 0;
  unsigned long long edges = 0, visits = 0;
  __shared__ SoloShared solo;
  if (!phase_g<G>(w, c, iterations, edges, visits, solo)) return;
  const int new_buf = s.ctl->cur_buf ^ (iterations & 1);
  phase_h(w, c, new_buf);
  edges = static_cast<unsigned long long>(warp_sum_ll(static_cast<long long>(edges)));
  visits = static_cast<unsigned long long>(warp_sum_ll(static_cast<long long>(visits)));
  if (c.lane == 0) {
    if (edges) atomicAdd(&s.bc->aff_edges, edges);
    if (visits) atomicAdd(&s.bc->front_visits, visits);
  }
  if (!grid_sync(bar, err, to)) return;

  if (blockIdx.x == 0 && threadIdx.x == 0) {
    dlp_batch_stats st;
    memset(&st, 0, sizeof(st));
    st.batch = a.batch;
    st.iterations = iterations;
    st.num_components = comp_path ? s.bc->num_comp : 0;
    st.num_sub_edges = comp_path ? 2 * s.bc->num_kept : 0;
    st.hook_edges = a.spec ? 2 * hook_count : hook_count;  // directed edges of G' (spec)
    st.hook_rounds = rounds;
    st.seed_frontier = s.bc->seed_frontier;
    st.seed_marks = s.bc->num_seeds;
    st.affected_edges = static_cast<int64_t>(s.bc->aff_edges);
    st.frontier_visits = static_cast<int64_t>(s.bc->front_visits);
    st.correct = s.ctl->correct;
    st.total = s.ctl->total;
    st.accuracy = st.total > 0 ? static_cast<float>(st.correct) / static_cast<float>(st.total) : 1.0f;
    st.status = DLP_OK;
    st.init_branch = comp_path ? 1 : (a.I > 0 ? 2 : 0);
    st.hook_truncated = (!a.spec && comp_path && 2 * s.bc->num_kept > a.E) ? 1 : 0;
    st.dirty_rows = s.bc->num_dirty;
    st.dirty_entries = static_cast<int64_t>(s.bc->dirty_entries);
    *s.stats_slot = st;
    s.ctl->cur_buf = new_buf;
    s.ctl->stamp_base = base + 1u + static_cast<unsigned>(iterations) + 1u;
  }
}

template __global__ void batch_kernel<4>(DevState, BatchArgs);
template __global__ void batch_kernel<8>(DevState, BatchArgs);
template __global__ void batch_kernel<16>(DevState, BatchArgs);
template __global__ void batch_kernel<32>(DevState, BatchArgs);

const void *batch_kernel_ptr(int lanes) {
  switch (lanes) {
    case 4: return reinterpret_cast<const void *>(&batch_kernel<4>);
    case 8: return reinterpret_cast<const void *>(&batch_kernel<8>);
    case 16: return reinterpret_cast<const void *>(&batch_kernel<16>);
    case 32: return reinterpret_cast<const void *>(&batch_kernel<32>);
    default: return nullptr;
  }
}

}  // namespace session
}  // namespace dlp
