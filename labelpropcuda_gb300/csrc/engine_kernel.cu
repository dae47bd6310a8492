// The multi-graph batch engine kernel (see engine.cuh). One cooperative
// persistent launch applies one batch to each listed graph; the phases and
// their arithmetic are the single-graph ones (session_kernel.cuh), each walking
// a work list flattened over all graphs.
//
// Arithmetic that must agree bit for bit with the CPU oracle:
//   * a row's weighted average follows the reference's summation order (slot
//     t of a 256-slot block accumulates entries t, t+256, ...; weight by add,
//     weighted label by FMA; tree with strides 128..1,
//     src/iterativePropagation.cu:126-150). A row of at most 32 entries only
//     adds +0 at strides 128..32, so a group of G lanes holding slots lane+G*r
//     reproduces it exactly; longer rows take a warp holding lane+32*j.
//   * division is IEEE round-to-nearest (__fdiv_rn; or, with
//     dlp_config.arithmetic = 1, the reference's fast-math division);
//     built with -fmad=false.
//   * supernode weights are exact 32.32 fixed-point sums (order independent).
#include "engine.cuh"

namespace dlp {
namespace engine {
namespace {

using session::BatchArgs;
using session::BatchCounters;
using session::DevState;
using session::kBlock;
using session::kMaxHookRounds;
using session::kNarrowMax;
using session::kRecordIters;
using session::kRowGroup;

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

__device__ __forceinline__ bool in_range(int v, int n) {
  return static_cast<unsigned>(v) < static_cast<unsigned>(n);
}

// One graph's state and batch as a phase sees them.
struct GV {
  const DevState &s;
  const BatchArgs &a;
  unsigned cur;  // this batch's stamp for deleted / GT / dirty marks
  unsigned g0;   // this batch's first frontier stamp

  __device__ bool inserted_now(int v) const {
    const int p = s.local[v];
    return p >= 0 && p < a.I && a.ins[p] == v;
  }
  // ref: a vertex inserted and deleted in one batch is DELETED for that batch
  __device__ bool dev_deleted(int v) const { return !a.spec && s.del_stamp[v] == cur; }
  // live in the host rebuild of this batch (src/dynLP.cu:143-157)
  __device__ bool live(int v) const {
    if (s.status[v] == kDeleted) return false;
    if (s.batch_map) {
      const int m = s.batch_map[v];
      if (m < 0 || m > a.batch) return false;
    }
    return true;
  }
  __device__ bool comp_path() const { return a.spec ? (a.I > 0) : (a.I > 0 && a.E > 0); }
};

__device__ __forceinline__ GV view(const EngineArgs &e, int g) {
  const GraphRec &r = e.recs[g];
  return GV{r.st, r.ba, static_cast<unsigned>(r.ba.seq) + 1u, r.st.ctl->stamp_base + 1u};
}

// ----------------------------------------------------------- warp helpers --
// Reserves one slot per predicated lane in the list whose counter is `count`;
// lanes of one warp may target different counters (different graphs).
// Called by all 32 lanes. Returns the slot, or -1 for lanes without pred.
__device__ __forceinline__ int reserve_keyed(bool pred, int *count) {
  const unsigned act = __ballot_sync(0xffffffffu, pred);
  if (!pred) return -1;
  const unsigned peers = __match_any_sync(act, reinterpret_cast<unsigned long long>(count));
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(count, __popc(peers));
  base = __shfl_sync(peers, base, leader);
  return base + __popc(peers & ((1u << lane) - 1u));
}

__device__ __forceinline__ void append_keyed(bool pred, int value, int *list, int *count) {
  const int slot = reserve_keyed(pred, count);
  if (slot >= 0) list[slot] = value;
}

__device__ __forceinline__ void append_back_keyed(bool pred, int value, int *list, int cap, int *count) {
  const int slot = reserve_keyed(pred, count);
  if (slot >= 0) list[cap - 1 - slot] = value;
}

// Adds v into *dst once per group of lanes sharing dst (all 32 lanes call).
__device__ __forceinline__ void add_keyed(bool pred, unsigned v, unsigned long long *dst) {
  const unsigned act = __ballot_sync(0xffffffffu, pred && v != 0);
  if (!(pred && v != 0)) return;
  const unsigned peers = __match_any_sync(act, reinterpret_cast<unsigned long long>(dst));
  const unsigned sum = __reduce_add_sync(peers, v);
  if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(dst, static_cast<unsigned long long>(sum));
}

// ------------------------------------------------------ flattened lists ----
// Exclusive prefix of per-graph counts in shared memory (all block threads
// call; the counts must read the same global values in every block).
template <class F>
__device__ int flat_build(int *pref, int ng, F count) {
  __shared__ int s_warp[kBlock / 32];
  __syncthreads();
  if (ng == 1) {
    if (threadIdx.x == 0) {
      pref[0] = 0;
      pref[1] = count(0);
    }
    __syncthreads();
    return pref[1];
  }
  constexpr int kPer = (kMaxGraphs + kBlock - 1) / kBlock;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int vals[kPer];
  int local = 0;
  const int start = threadIdx.x * kPer;
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    const int g = start + j;
    vals[j] = g < ng ? count(g) : 0;
    local += vals[j];
  }
  int incl = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int x = lane < kBlock / 32 ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane < kBlock / 32) s_warp[lane] = x;
  }
  __syncthreads();
  int run = incl - local + (warp > 0 ? s_warp[warp - 1] : 0);
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    const int g = start + j;
    if (g < ng) pref[g] = run;
    run += vals[j];
  }
  if (threadIdx.x == kBlock - 1) pref[ng] = run;
  __syncthreads();
  return pref[ng];
}

// Largest g with pref[g] <= item: the graph that owns work item `item`.
__device__ __forceinline__ int locate(const int *pref, int ng, int item) {
  int lo = 0, hi = ng - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pref[mid] <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Group-of-kRowGroup items over a flattened list; every lane of a warp runs
// the same number of iterations so warp collectives stay legal.
template <class F>
__device__ __forceinline__ void flat_groups(const Ctx &c, const int *pref, int ng, int total, F fn) {
  constexpr int GPW = 32 / kRowGroup;
  const int grp = c.lane / kRowGroup, gl = c.lane & (kRowGroup - 1);
  for (int base = c.gwarp * GPW; base < total; base += c.nwarps * GPW) {
    const int item = base + grp;
    const bool valid = item < total;
    const int g = valid ? locate(pref, ng, item) : 0;
    fn(g, valid ? item - pref[g] : 0, valid, gl, grp);
  }
}

// Per-thread items over a flattened list, warp-uniform trip count.
template <class F>
__device__ __forceinline__ void flat_threads(const Ctx &c, const int *pref, int ng, int total, F fn) {
  for (int base = c.gwarp * 32; base < total; base += c.nwarps * 32) {
    const int item = base + c.lane;
    const bool valid = item < total;
    const int g = valid ? locate(pref, ng, item) : 0;
    fn(g, valid ? item - pref[g] : 0, valid);
  }
}

// Seed mark: the batch's first stamp; the first mark appends to the seed list.
__device__ __forceinline__ void seed_mark(const GV &w, bool cand, int v) {
  bool first = false;
  if (cand) first = atomicMax(&w.s.front_stamp[v], w.g0) < w.g0;
  append_keyed(first, v, w.s.seed_list, &w.s.bc->num_seeds);
}

// Frontier append into set `set` (narrow rows from the front, wide from the
// back) and, the first time in this batch, into the touched list.
__device__ __forceinline__ void frontier_append(const GV &w, bool pred, bool first, int v, int set) {
  const DevState &s = w.s;
  bool wide = false;
  if (pred) wide = s.act_len[v] > kNarrowMax;
  int *list = s.flist + static_cast<size_t>(set) * s.n;
  append_keyed(pred && !wide, v, list, &s.bc->front_count[set][0]);
  append_back_keyed(pred && wide, v, list, s.n, &s.bc->front_count[set][1]);
  append_keyed(first, v, s.touched + static_cast<size_t>(w.a.seq & 1) * s.n, &s.ctl->touched_count[w.a.seq & 1]);
}

// ---------------------------------------------------------------- phase A ---
// Position map, stamps, input validation, label-buffer re-sync at the vertices
// the previous batch's propagation wrote (both buffers start a batch equal,
// src/dynLP.cu:519 and src/iterativePropagation.cu:268-270).
__device__ void phase_a(const EngineArgs &e, const Ctx &c, int *pref) {
  const int ng = e.ng_new;
  auto prev_touched = [&](int g) {
    const GraphRec &r = e.recs[g];
    return r.ba.seq > 0 ? r.st.ctl->touched_count[(r.ba.seq - 1) & 1] : 0;
  };
  const int total = flat_build(pref, ng, [&](int g) {
    const BatchArgs &a = e.recs[g].ba;
    return a.I + a.D + a.G + a.E + prev_touched(g);
  });
  int bad = 0;
  for (int item = c.gtid; item < total; item += c.nthreads) {
    const int g = locate(pref, ng, item);
    int i = item - pref[g];
    const GV w = view(e, g);
    const DevState &s = w.s;
    const BatchArgs &a = w.a;
    const int n = s.n;
    if (i < a.I) {
      const int v = a.ins[i];
      if (!in_range(v, n)) { bad = 1; continue; }
      s.local[v] = i;
      s.par[i] = i;
      s.acc[2 * i] = 0;
      s.acc[2 * i + 1] = 0;
      if (a.record) s.rec_minid[i] = 0x7fffffff;
      continue;
    }
    i -= a.I;
    if (i < a.D) {
      const int v = a.del[i];
      if (!in_range(v, n)) { bad = 1; continue; }
      if (a.spec) s.del_pre[i] = s.status[v];
      s.del_stamp[v] = w.cur;
      continue;
    }
    i -= a.D;
    if (i < a.G) {
      const int v = a.gt_ids[i];
      if (!in_range(v, n)) { bad = 1; continue; }
      s.gt_stamp[v] = w.cur;
      continue;
    }
    i -= a.G;
    if (i < a.E) {
      if (!in_range(a.es[i], n) || !in_range(a.ed[i], n)) bad = 1;
      continue;
    }
    i -= a.E;
    const int cb = s.ctl->cur_buf;
    const int v = s.touched[static_cast<size_t>((a.seq - 1) & 1) * n + i];
    (cb ? s.lab0 : s.lab1)[v] = (cb ? s.lab1 : s.lab0)[v];
  }
  for (int g = c.gtid; g < ng; g += c.nthreads) {
    const GraphRec &r = e.recs[g];
    r.st.ctl->touched_count[r.ba.seq & 1] = 0;
  }
  if (bad) atomicCAS(&e.ectl->err, 0, DLP_ERR_INVALID_ARGUMENT);
}

// ---------------------------------------------------------------- phase B ---
// Host-status update (ref: delete, insert, then ground truth,
// src/dynLP.cu:117-130; spec: deletions win) and dirty-row marking.
__device__ void phase_b(const EngineArgs &e, const Ctx &c, int *pref) {
  const int ng = e.ng_new;
  int total = flat_build(pref, ng, [&](int g) {
    const BatchArgs &a = e.recs[g].ba;
    return a.D + a.I + a.G;
  });
  for (int item = c.gtid; item < total; item += c.nthreads) {
    const int g = locate(pref, ng, item);
    int i = item - pref[g];
    const GV w = view(e, g);
    const DevState &s = w.s;
    const BatchArgs &a = w.a;
    if (i < a.D) {
      const int v = a.del[i];
      if (a.spec || (!w.inserted_now(v) && s.gt_stamp[v] != w.cur)) s.status[v] = kDeleted;
      continue;
    }
    i -= a.D;
    if (i < a.I) {
      const int v = a.ins[i];
      if (s.gt_stamp[v] == w.cur) continue;
      if (a.spec && s.del_stamp[v] == w.cur) continue;
      s.status[v] = kActive;
      continue;
    }
    i -= a.I;
    const int v = a.gt_ids[i];
    const float l = a.gt_lab[i];
    s.gt[v] = l < 0.5f ? 0 : 1;
    s.nmeta[v] = s.act_len[v] > kNarrowMax ? 2 : 0;  // not markable any more
    s.lab0[v] = l;
    s.lab1[v] = l;
    if (!(a.spec && s.del_stamp[v] == w.cur)) s.status[v] = kGroundTruth;
  }
  // Rows whose live content can change: every changed vertex and its
  // full-graph neighbours; the previous batch's deletions give a same-batch
  // insert+delete (ref) its row back.
  total = flat_build(pref, ng, [&](int g) {
    const BatchArgs &a = e.recs[g].ba;
    return a.D + a.I + a.PD + a.G;
  });
  flat_groups(c, pref, ng, total, [&](int g, int k, bool valid, int gl, int) {
    const GV w = view(e, g);
    const DevState &s = w.s;
    const BatchArgs &a = w.a;
    int x = -1;
    if (valid) {
      if (k < a.D) x = a.del[k];
      else if ((k -= a.D) < a.I) x = a.ins[k];
      else if ((k -= a.I) < a.PD) x = a.prev_del[k];
      else x = a.gt_ids[k - a.PD];
    }
    const int rs = valid ? s.full_row[x] : 0;
    const int len = valid ? s.full_row[x + 1] - rs : 0;
    const int maxlen = __reduce_max_sync(0xffffffffu, len + 1);  // +1: the vertex itself
    for (int off = 0; off < maxlen; off += kRowGroup) {
      const int ee = off + gl - 1;  // -1: x itself
      int v = -1;
      if (valid && ee < len) v = ee < 0 ? x : s.full_adj[rs + ee].x;
      bool first = false;
      if (v >= 0) first = atomicMax(&s.dirty_stamp[v], w.cur) < w.cur;
      append_keyed(first, v, s.dirty_list, &s.bc->num_dirty);
    }
  });
}

// ---------------------------------------------------------------- phase C ---
// Live-row compaction, deletion marks and the tau filter.
__device__ void phase_c(const EngineArgs &e, const Ctx &c, int *pref) {
  const int ng = e.ng_new;
  int total = flat_build(pref, ng, [&](int g) { return e.recs[g].st.bc->num_dirty; });
  flat_groups(c, pref, ng, total, [&](int g, int item, bool valid, int gl, int grp) {
    const GV w = view(e, g);
    const DevState &s = w.s;
    int u = 0, rs = 0, len = 0;
    bool keep_row = false, del_row = false;
    if (valid) {
      u = s.dirty_list[item];
      keep_row = w.live(u);
      rs = s.full_row[u];
      len = keep_row ? s.full_row[u + 1] - rs : 0;
      del_row = keep_row && w.dev_deleted(u);
    }
    add_keyed(valid && gl == 0, static_cast<unsigned>(len), &s.bc->dirty_entries);
    const int maxlen = __reduce_max_sync(0xffffffffu, len);
    const unsigned gmask = ((1u << kRowGroup) - 1u) << (grp * kRowGroup);
    int pos = 0;
    for (int off = 0; off < maxlen; off += kRowGroup) {
      const int ee = off + gl;
      bool keep = false;
      int2 ent = make_int2(-1, 0);
      if (ee < len) {
        ent = s.full_adj[rs + ee];
        keep = ent.x >= 0 && w.live(ent.x);
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep) & gmask;
      if (keep) {
        const int rank = __popc(m & ((1u << c.lane) - 1u));
        int col = ent.x;
        // soft delete (src/sparsifySubgraph.cu:78,108): entries of a row deleted
        // this batch and entries pointing at such a vertex
        if (del_row || w.dev_deleted(col)) col = -1;
        s.act_adj[rs + pos + rank] = make_int2(col, ent.y);
      }
      // neighbours of a deleted vertex's live row are affected
      // (src/sparsifySubgraph.cu:71-76; empty unless inserted this batch)
      seed_mark(w, keep && del_row, ent.x);
      pos += __popc(m);
    }
    if (valid && gl == 0) {
      const int len = keep_row ? pos : 0;
      s.act_len[u] = len;
      s.rowinfo[u] = make_int2(rs, len);
      s.nmeta[u] = static_cast<uint8_t>((s.gt[u] < 0 ? 1 : 0) | (len > kNarrowMax ? 2 : 0));
    }
  });

  // spec: neighbours of every deleted vertex that was live before this batch's
  // deletions, in the adjacency before the deletion
  total = flat_build(pref, ng, [&](int g) {
    const BatchArgs &a = e.recs[g].ba;
    return a.spec ? a.D : 0;
  });
  if (total > 0)
    flat_groups(c, pref, ng, total, [&](int g, int item, bool valid, int gl, int) {
      const GV w = view(e, g);
      const DevState &s = w.s;
      int x = 0;
      bool was = false;
      if (valid) {
        x = w.a.del[item];
        was = s.del_pre[item] != kDeleted || w.inserted_now(x) || s.gt_stamp[x] == w.cur;
        if (was && s.batch_map) {
          const int m = s.batch_map[x];
          was = m >= 0 && m <= w.a.batch;
        }
      }
      const int rs = was ? s.full_row[x] : 0;
      const int len = was ? s.full_row[x + 1] - rs : 0;
      const int maxlen = __reduce_max_sync(0xffffffffu, len);
      for (int off = 0; off < maxlen; off += kRowGroup) {
        const int ee = off + gl;
        const int v = ee < len ? s.full_adj[rs + ee].x : -1;
        seed_mark(w, v >= 0 && w.live(v), v);
      }
    });

  // Tau filter over each batch's raw edges, four per lane (int4/float4 loads
  // when the arrays are 16-byte aligned): positions for the components step,
  // the kept new-new edges, and the endpoint marks.
  total = flat_build(pref, ng, [&](int g) {
    const GV w = view(e, g);
    return w.comp_path() ? (w.a.E + 3) >> 2 : 0;
  });
  flat_threads(c, pref, ng, total, [&](int g, int q, bool valid) {
    const GV w = view(e, g);
    const DevState &s = w.s;
    const BatchArgs &a = w.a;
    int sv[4] = {0, 0, 0, 0}, dv[4] = {0, 0, 0, 0};
    float wv[4] = {0.f, 0.f, 0.f, 0.f};
    int nv = 0;
    if (valid) {
      const int base = q * 4;
      nv = min(4, a.E - base);
      const bool vec = nv == 4 && ((reinterpret_cast<uintptr_t>(a.es) | reinterpret_cast<uintptr_t>(a.ed) |
                                    reinterpret_cast<uintptr_t>(a.ew)) & 15u) == 0;
      if (vec) {
        const int4 s4 = reinterpret_cast<const int4 *>(a.es)[q];
        const int4 d4 = reinterpret_cast<const int4 *>(a.ed)[q];
        const float4 w4 = reinterpret_cast<const float4 *>(a.ew)[q];
        sv[0] = s4.x; sv[1] = s4.y; sv[2] = s4.z; sv[3] = s4.w;
        dv[0] = d4.x; dv[1] = d4.y; dv[2] = d4.z; dv[3] = d4.w;
        wv[0] = w4.x; wv[1] = w4.y; wv[2] = w4.z; wv[3] = w4.w;
      } else {
        for (int j = 0; j < nv; ++j) {
          sv[j] = a.es[base + j];
          dv[j] = a.ed[base + j];
          wv[j] = a.ew[base + j];
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const bool ok = valid && j < nv;
      int ls = -1, ld = -1;
      bool kept = false;
      if (ok) {
        ls = w.inserted_now(sv[j]) ? s.local[sv[j]] : -1;
        ld = w.inserted_now(dv[j]) ? s.local[dv[j]] : -1;
        kept = wv[j] > a.tau && ls >= 0 && ld >= 0;
        s.lsrc[q * 4 + j] = ls;
        s.ldst[q * 4 + j] = ld;
      }
      // kept new-new edge (src/sparsifySubgraph.cu:133,165-174)
      const int k = reserve_keyed(kept, &s.bc->num_kept);
      if (k >= 0) {
        s.sub_pairs[2 * k] = sv[j];
        s.sub_pairs[2 * k + 1] = dv[j];
        s.sub_local[2 * k] = ls;
        s.sub_local[2 * k + 1] = ld;
      }
      if (!a.spec) {
        // ref: endpoints of edges with w > tau, clipped to ids below the
        // inserted count (src/sparsifySubgraph.cu:259-263 with :177-178)
        const bool heavy = ok && wv[j] > a.tau;
        seed_mark(w, heavy && sv[j] < a.I, sv[j]);
        seed_mark(w, heavy && dv[j] < a.I, dv[j]);
      } else {
        seed_mark(w, ok && w.live(sv[j]), sv[j]);
        seed_mark(w, ok && w.live(dv[j]), dv[j]);
      }
    }
  });

  // spec: every new non-ground-truth vertex is affected
  total = flat_build(pref, ng, [&](int g) {
    const BatchArgs &a = e.recs[g].ba;
    return a.spec ? a.I : 0;
  });
  if (total > 0)
    flat_threads(c, pref, ng, total, [&](int g, int i, bool valid) {
      const GV w = view(e, g);
      const int v = valid ? w.a.ins[i] : 0;
      seed_mark(w, valid && w.s.gt[v] < 0 && w.live(v), v);
    });
}

// ---------------------------------------------------------------- phase D ---
__device__ void phase_d_frontier(const EngineArgs &e, const Ctx &c, int *pref) {
  const int ng = e.ng_new;
  const int total = flat_build(pref, ng, [&](int g) { return e.recs[g].st.bc->num_seeds; });
  flat_threads(c, pref, ng, total, [&](int g, int i, bool valid) {
    const GV w = view(e, g);
    const DevState &s = w.s;
    int v = 0;
    bool ok = false;
    if (valid) {
      v = s.seed_list[i];
      // collect filter (src/iterativePropagation.cu:73-75)
      ok = s.status[v] == kActive && !w.dev_deleted(v) && s.gt[v] < 0;
    }
    frontier_append(w, ok, ok, v, 0);
    const int slot = reserve_keyed(ok, &s.bc->seed_frontier);
    if (slot >= 0 && w.a.record) s.rec_front0[slot] = v;
  });
}

// Edges the components step hooks: ref, the first min(numSubEdges, E) raw
// edges (src/dynLP.cu:437-440); spec, the kept new-new edges.
__device__ __forceinline__ int hook_count(const GV &w) {
  if (!w.comp_path()) return 0;
  const int kept = w.s.bc->num_kept;
  if (w.a.spec) return kept;
  return kept > 0 ? min(2 * kept, w.a.E) : 0;
}

// Shiloach-Vishkin rounds for every graph with edges to hook: hook (larger
// root under the smaller with atomicMin, src/connectedComponents.cu:79-100),
// then pointer jumping to the root (:108-121), until a hook pass of that
// graph changes nothing. -1 stands for a vertex that is not new this batch.
__device__ bool phase_d_sv(const EngineArgs &e, const Ctx &c, int *pref) {
  const int ng = e.ng_new;
  for (int r = 0; r < kMaxHookRounds; ++r) {
    auto active = [&](int g) {
      const BatchCounters *bc = e.recs[g].st.bc;
      return r == 0 || ld_relaxed_i32(&bc->hook_flag[r - 1]) != 0;
    };
    int total = flat_build(pref, ng, [&](int g) { return active(g) ? hook_count(view(e, g)) : 0; });
    if (total == 0) break;
    flat_threads(c, pref, ng, total, [&](int g, int i, bool valid) {
      bool changed = false;
      int *flag = nullptr;
      if (valid) {
        const GV w = view(e, g);
        const DevState &s = w.s;
        const int *A = w.a.spec ? s.sub_local : s.lsrc;
        const int *B = w.a.spec ? s.sub_local + 1 : s.ldst;
        const size_t stride = w.a.spec ? 2 : 1;
        const int x = A[i * stride], y = B[i * stride];
        const int rx = x < 0 ? -1 : s.par[x];
        const int ry = y < 0 ? -1 : s.par[y];
        if (rx != ry) {
          const int hi = max(rx, ry), lo = min(rx, ry);
          if (atomicMin(&s.par[hi], lo) != lo) changed = true;
        }
        flag = &s.bc->hook_flag[r];
      }
      if (changed) *flag = 1;
    });
    if (!grid_sync(&e.ectl->bar, &e.ectl->err, e.timeout_ns)) return false;
    total = flat_build(pref, ng, [&](int g) { return active(g) && hook_count(view(e, g)) > 0 ? e.recs[g].ba.I : 0; });
    for (int item = c.gtid; item < total; item += c.nthreads) {
      const int g = locate(pref, ng, item);
      const DevState &s = e.recs[g].st;
      const int i = item - pref[g];
      int p = s.par[i];
      while (p >= 0) {
        const int q = s.par[p];
        if (q == p) break;
        p = q;
      }
      s.par[i] = p;
    }
    if (!grid_sync(&e.ectl->bar, &e.ectl->err, e.timeout_ns)) return false;
  }
  return true;
}

// ---------------------------------------------------------------- phase E ---
// Component count and fixed-point supernode weights per component root
// (src/labelInitialization.cu:59-88).
__device__ void phase_e(const EngineArgs &e, const Ctx &c, int *pref) {
  const int ng = e.ng_new;
  auto count = [&](int g) {
    const GV w = view(e, g);
    return w.comp_path() ? w.a.I : 0;
  };
  int total = flat_build(pref, ng, count);
  flat_threads(c, pref, ng, total, [&](int g, int i, bool valid) {
    const GV w = view(e, g);
    const DevState &s = w.s;
    bool root = false;
    if (valid) {
      const int p = s.par[i];
      root = p == i;
      if (w.a.record && p >= 0) atomicMin(&s.rec_minid[p], w.a.ins[i]);
    }
    const int slot = reserve_keyed(root, &s.bc->num_comp);
    (void)slot;
  });
  flat_groups(c, pref, ng, total, [&](int g, int item, bool valid, int gl, int) {
    const GV w = view(e, g);
    const DevState &s = w.s;
    int rs = 0, len = 0, root = -1;
    if (valid) {
      root = s.par[item];
      const int u = w.a.ins[item];
      if (root >= 0) {
        rs = s.full_row[u];
        len = s.act_len[u];
      }
    }
    const int maxlen = __reduce_max_sync(0xffffffffu, len);
    long long q0 = 0, q1 = 0;
    for (int off = 0; off < maxlen; off += kRowGroup) {
      const int ee = off + gl;
      if (ee < len) {
        const int2 ent = s.act_adj[rs + ee];
        if (ent.x >= 0) {
          const int gc = s.gt[ent.x];
          const long long q = to_fixed(__int_as_float(ent.y));
          if (gc == 0) q0 += q;
          else if (gc == 1) q1 += q;
        }
      }
    }
#pragma unroll
    for (int o = kRowGroup / 2; o > 0; o >>= 1) {
      q0 += __shfl_down_sync(0xffffffffu, q0, o, kRowGroup);
      q1 += __shfl_down_sync(0xffffffffu, q1, o, kRowGroup);
    }
    if (valid && gl == 0 && root >= 0) {
      if (q0) atomicAdd(reinterpret_cast<unsigned long long *>(&s.acc[2 * root]), static_cast<unsigned long long>(q0));
      if (q1)
        atomicAdd(reinterpret_cast<unsigned long long *>(&s.acc[2 * root + 1]), static_cast<unsigned long long>(q1));
    }
  });
}

// ---------------------------------------------------------------- phase F ---
__device__ void phase_f(const EngineArgs &e, const Ctx &c, int *pref) {
  const int ng = e.ng_new;
  const int total = flat_build(pref, ng, [&](int g) { return e.recs[g].ba.I; });
  for (int item = c.gtid; item < total; item += c.nthreads) {
    const int g = locate(pref, ng, item);
    const int i = item - pref[g];
    const GV w = view(e, g);
    const DevState &s = w.s;
    const BatchArgs &a = w.a;
    const int u = a.ins[i];
    const bool comp = w.comp_path();
    float l;
    if (comp) {
      // src/labelInitialization.cu:99-142
      const int gc = s.gt[u];
      const int root = s.par[i];
      if (gc == 0) l = 0.0f;
      else if (gc == 1) l = 1.0f;
      else if (root < 0) l = 0.5f;
      else {
        const float w0 = from_fixed(s.acc[2 * root]);
        const float w1 = from_fixed(s.acc[2 * root + 1]);
        const float den = w0 + w1;
        l = den > 1e-10f ? quotient(w1, den, e.fast_div) : 0.5f;
      }
      s.lab0[u] = l;
      s.lab1[u] = l;
    } else if (s.gt_stamp[u] == w.cur && s.gt[u] >= 0) {
      // new vertices without new edges (src/dynLP.cu:482-504): this batch's
      // ground truth keeps the label set in phase B, everything else 0.5
      l = s.lab0[u];
    } else {
      l = 0.5f;
      s.lab0[u] = l;
      s.lab1[u] = l;
    }
    if (a.record) {
      s.rec_init[i] = l;
      const int root = comp ? s.par[i] : -1;
      s.rec_root[i] = root < 0 ? -1 : s.rec_minid[root];
    }
  }
}

// ---------------------------------------------------------------- phase G ---
// One row of at most 32 live entries by a group of G lanes; calls
// mark(cand, v) for each slot and for u itself, on every lane.
// cand[] receives what a changed row marks (src/iterativePropagation.cu:200-216):
// its non-deleted, non-ground-truth neighbours (cand[0..R)) and the vertex
// itself (cand[R]), -1 where nothing is marked; bit r of wide_bits is set when
// cand[r]'s live row is longer than 32 entries. Every load that depends only
// on the row (own label, neighbour labels, classes and row lengths) is issued
// before the row's sum is formed, so a row costs three dependent memory round
// trips (list entry, row, neighbours) before its marks.
template <int G>
__device__ __forceinline__ void narrow_row(const DevState &s, const float *src, float *dst, float delta, bool fast,
                                           int u, bool valid, int gl, int &len_out, int (&cand)[32 / G + 1],
                                           unsigned &wide_bits) {
  constexpr int R = 32 / G;
  int rs = 0, len = 0;
  float old = 0.0f;
  if (valid) {
    const int2 ri = s.rowinfo[u];
    rs = ri.x;
    len = ri.y;
    if (gl == 0) old = src[u];
  }
  float sw[R], sl[R];
  int vv[R];
  unsigned wb = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int ee = gl + G * r;
    sw[r] = 0.0f;
    sl[r] = 0.0f;
    vv[r] = -1;
    if (ee < len) {
      const int2 ent = s.act_adj[rs + ee];
      if (ent.x >= 0) {
        const float wt = __int_as_float(ent.y);
        sw[r] = wt;                               // 0 + w
        sl[r] = __fmaf_rn(wt, src[ent.x], 0.0f);  // fma(w, F_v, 0)
        const unsigned meta = s.nmeta[ent.x];
        if (meta & 1u) vv[r] = ent.x;
        if (meta & 2u) wb |= 1u << r;
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
    const float nl = updated_label(tw, tl, old, fast);
    dst[u] = nl;
    changed = fabsf(nl - old) > delta;
  }
  changed = __shfl_sync(0xffffffffu, changed, 0, G);
  len_out = len;
#pragma unroll
  for (int r = 0; r < R; ++r) cand[r] = changed ? vv[r] : -1;
  cand[R] = (changed && gl == 0) ? u : -1;
  if (len > kNarrowMax) wb |= 1u << R;
  wide_bits = changed ? wb : 0u;
}

// Marks of one G-lane group (one row, one graph): every stamp atomic is
// issued before any result is used, then each of the three lists (narrow
// rows from the front of set `set`, wide rows from its back, the batch's
// touched list) gets one reservation for the whole group. The marked set is
// the same as marking one candidate at a time; only the order of the list
// entries differs, and nothing depends on that order.
template <int G>
__device__ __forceinline__ void group_mark(const GV &w, const int (&cand)[32 / G + 1], unsigned wide_bits,
                                           unsigned stamp, int set, int gl) {
  constexpr int C = 32 / G + 1;
  const DevState &s = w.s;
  unsigned old[C];
#pragma unroll
  for (int r = 0; r < C; ++r) old[r] = cand[r] >= 0 ? atomicMax(&s.front_stamp[cand[r]], stamp) : stamp;
  int nn = 0, nw = 0, nf = 0;
#pragma unroll
  for (int r = 0; r < C; ++r) {
    if (old[r] < stamp) {
      if ((wide_bits >> r) & 1u) ++nw;
      else ++nn;
    }
    if (old[r] < w.g0) ++nf;
  }
  // counts packed 10 bits each (a group marks at most 64 vertices)
  const int mine = nn | (nw << 10) | (nf << 20);
  int incl = mine;
#pragma unroll
  for (int o = 1; o < G; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o, G);
    if (gl >= o) incl += t;
  }
  const int tot = __shfl_sync(0xffffffffu, incl, G - 1, G);
  int bn = 0, bw = 0, bf = 0;
  if (gl == G - 1 && tot != 0) {
    const int tn = tot & 1023, tw = (tot >> 10) & 1023, tf = tot >> 20;
    if (tn) bn = atomicAdd(&s.bc->front_count[set][0], tn);
    if (tw) bw = atomicAdd(&s.bc->front_count[set][1], tw);
    if (tf) bf = atomicAdd(&s.ctl->touched_count[w.a.seq & 1], tf);
  }
  bn = __shfl_sync(0xffffffffu, bn, G - 1, G);
  bw = __shfl_sync(0xffffffffu, bw, G - 1, G);
  bf = __shfl_sync(0xffffffffu, bf, G - 1, G);
  if (mine == 0) return;
  const int excl = incl - mine;
  int on = bn + (excl & 1023), ow = bw + ((excl >> 10) & 1023), of = bf + (excl >> 20);
  int *list = s.flist + static_cast<size_t>(set) * s.n;
  int *touched = s.touched + static_cast<size_t>(w.a.seq & 1) * s.n;
#pragma unroll
  for (int r = 0; r < C; ++r) {
    if (old[r] < stamp) {
      if ((wide_bits >> r) & 1u) list[s.n - 1 - ow++] = cand[r];
      else list[on++] = cand[r];
    }
    if (old[r] < w.g0) touched[of++] = cand[r];
  }
}

// One row of any length by a whole warp: 256 slots held as lane + 32*j.
template <class Mark>
__device__ __forceinline__ void wide_row(const DevState &s, const float *src, float *dst, float delta, bool fast,
                                         int u, int lane, Mark mark) {
  const int2 ri = s.rowinfo[u];
  const int rs = ri.x;
  const int len = ri.y;
  float sw[8], sl[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) sw[j] = sl[j] = 0.0f;
  for (int p = 0; p < len; p += 256) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int ee = p + j * 32 + lane;
      if (ee < len) {
        const int2 ent = s.act_adj[rs + ee];
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
    const float nl = updated_label(tw, tl, old, fast);
    dst[u] = nl;
    changed = fabsf(nl - old) > delta;
  }
  changed = __shfl_sync(0xffffffffu, changed, 0);
  if (changed) {
    for (int e0 = 0; e0 < len; e0 += 32) {
      const int ee = e0 + lane;
      const int v = ee < len ? s.act_adj[rs + ee].x : -1;
      mark(v >= 0 && s.gt[v] < 0, v);
    }
    mark(lane == 0, u);
  }
}

// A graph takes part in the launch's pass k (its own pass k + pass0) while its
// frontier is not empty and its pass is below max_iter; passes counts the
// passes it ran.
__device__ __forceinline__ bool graph_in_pass(const GraphRec &r, int k, int &nn, int &nw) {
  const BatchCounters *bc = r.st.bc;
  const int kg = k + r.ba.pass0;
  nn = ld_relaxed_i32(&bc->front_count[kg % 3][0]);
  nw = ld_relaxed_i32(&bc->front_count[kg % 3][1]);
  return nn + nw > 0 && kg < r.ba.max_iter;
}

// True once the launch's time slice has run out (checked by thread 0 of block
// 0 only, which recorded the launch's start).
__device__ __forceinline__ bool slice_over(const EngineArgs &e) {
  return e.slice_ns != 0 && global_timer_ns() - e.ectl->t_launch > e.slice_ns;
}

// A stop request for pass k of this launch (EngineCtl::sub_stop, slice_stop).
__device__ __forceinline__ unsigned long long stop_code(const EngineArgs &e, int k) {
  return (static_cast<unsigned long long>(static_cast<unsigned>(e.tag)) << 32) | static_cast<unsigned>(k);
}

// Solo mode: when all graphs' frontiers together are small, block 0 runs the
// passes alone with __syncthreads() between them while the other blocks wait
// at the next grid barrier. The vertices the passes touch are held in shared
// memory for the whole stint: a vertex table (both label buffers, row
// length, mark) for the frontier vertices and their neighbours, and a row pool with
// each frontier row's entries as (table slot, weight). A row is loaded from
// HBM the first time its vertex is in the frontier; afterwards a pass touches
// only shared memory. Labels of vertices outside the frontier cannot change
// during the stint, so loading them once is exact; every label written goes
// back to HBM when the stint ends. Passes and arithmetic are those of the
// grid path (same slot order in every row, same summation tree).
constexpr int kVT = 2048;          // vertex-table slots (power of two), at most three quarters in use
#ifndef DLP_SOLO_VT_USE
#define DLP_SOLO_VT_USE (3 * kVT / 4)
#endif
constexpr int kVTUse = DLP_SOLO_VT_USE;  // slots in use at most (linear probing stays short below this)
constexpr int kRP = 4096;          // row-pool entries
// frontier capacity: a list holds distinct vertex-table slots, so it can never
// need more entries than the table has slots in use
constexpr int kSoloList = kVTUse;
static_assert(kSoloList >= kVTUse, "a one-block frontier list must hold every slot in use");
static_assert(kSoloEntryMax <= kVTUse && kSoloEntryMax <= kSoloList,
              "a one-block stint starts by putting the whole frontier into the vertex table and list 0");
constexpr int kSoloMaxPasses = 65000;  // per stint, so that per-slot visit counts fit 16 bits
constexpr unsigned long long kSoloBudgetNs = 100000000ull;
constexpr unsigned long long kEmptyKey = ~0ull;
constexpr unsigned char kWideLen = 255;
constexpr unsigned short kNoRow = 0xffff;
#ifndef DLP_SOLO_LANES
#define DLP_SOLO_LANES 4
#endif
constexpr int kSoloG = DLP_SOLO_LANES;  // lanes per row in the one-block passes (build-time choice)

struct SoloCache {
  unsigned long long key[kVT];   // (graph << 32) | vertex, kEmptyKey = free
  float lab[2][kVT];             // the graph's physical buffers 0 and 1
  int mark[kVT];                 // last pass (+1) that put the slot in the next frontier; INT_MAX: ground truth
  unsigned short row[kVT];       // row-pool offset, kNoRow = not loaded
  unsigned short visits[kVT];    // passes of the stint that updated the slot
  int2 rp[kRP];                  // {neighbour slot or -1, weight bits}
  unsigned short list[2][kSoloList];
  unsigned short graph[kVT];
  unsigned char len[kVT];        // live row length, kWideLen when longer than 32
  unsigned char flags[kVT];      // bit0 written, bit1 in a frontier, bit2 buffer read at stint pass 0
  int lastpass[kMaxGraphs];      // last launch pass each graph took part in during the stint
  // Per list, indexed by stint pass % 3: the list read by pass j is filled
  // during pass j - 1 and its counters are cleared during pass j + 1, so a
  // thread reading them at the top of pass j never races a writer.
  int cnt[3];                    // entries
  int need[3];                   // row entries still to load
  int wide[3];                   // holds a row longer than 32 entries
  int used;                      // vertex-table slots in use
  int rp_top;                    // row-pool entries in use
  int stop_at;                   // stint pass at which a time budget stops the stint
  int stop_slice;                // that budget was the launch's time slice
  int team_end;                  // first pass a team stint did not run
};

__device__ __forceinline__ unsigned mix64(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  return static_cast<unsigned>(x);
}

// Slot of (g, v) in the vertex table, inserting (and loading from HBM) when
// absent. The caller keeps the table at most three quarters full.
__device__ __forceinline__ int vt_slot(SoloCache &c, const EngineArgs &e, int g, int v) {
  const unsigned long long key = (static_cast<unsigned long long>(g) << 32) | static_cast<unsigned>(v);
  unsigned h = mix64(key) & (kVT - 1);
  for (int probe = 0; probe < kVT; ++probe) {
    const unsigned long long prev = atomicCAS(&c.key[h], kEmptyKey, key);
    if (prev == kEmptyKey) {
      const DevState &s = e.recs[g].st;
      c.lab[0][h] = s.lab0[v];
      c.lab[1][h] = s.lab1[v];
      const int len = s.act_len[v];
      c.len[h] = len > kNarrowMax ? kWideLen : static_cast<unsigned char>(len);
      c.graph[h] = static_cast<unsigned short>(g);
      c.flags[h] = static_cast<unsigned char>(((s.ctl->cur_buf ^ e.recs[g].ba.pass0) & 1) << 2);
      c.row[h] = kNoRow;
      c.visits[h] = 0;
      c.mark[h] = s.gt[v] < 0 ? -1 : 0x7fffffff;  // a ground-truth slot is never marked
      atomicAdd(&c.used, 1);
      return static_cast<int>(h);
    }
    if (prev == key) return static_cast<int>(h);
    h = (h + 1) & (kVT - 1);
  }
  return -1;  // not reached: the table always has free slots
}

// One pass of the one-block mode over the rows of `cur` (cnt entries), G lanes
// per row, by the block's first NW warps: every row from shared memory, marks
// into `next` and the counters of list nq. G and NW only set how the rows are
// spread over the threads; the arithmetic and the marked set do not depend on
// them.
template <int G, int NW>
__device__ __forceinline__ void solo_rows(const EngineArgs &e, SoloCache &c, const unsigned short *cur,
                                          unsigned short *next, int cnt, int nq, int k, bool rec_any) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int R = 32 / G;
  constexpr int GPW = 32 / G;
  const int grp = lane / G, gl = lane & (G - 1);

  for (int base = warp * GPW; base < cnt; base += NW * GPW) {
    const int item = base + grp;
    const bool valid = item < cnt;
    const int su = valid ? cur[item] : 0;
    const int len = valid ? c.len[su] : 0;
    const int off = valid ? c.row[su] : 0;
    const int src = valid ? (((c.flags[su] >> 2) ^ k) & 1) : 0;
    float sw[R], sl[R];
    int vv[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int ee = gl + G * r;
      sw[r] = 0.0f;
      sl[r] = 0.0f;
      vv[r] = -1;
      if (ee < len) {
        const int2 ent = c.rp[off + ee];
        vv[r] = ent.x;
        if (ent.x >= 0) {
          const float wt = __int_as_float(ent.y);
          sw[r] = wt;
          sl[r] = __fmaf_rn(wt, c.lab[src][ent.x], 0.0f);
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
      // nothing here reads the graph's record in global memory: delta is
      // the engine's, and the pass offset is added at hand-back
      const int g = c.graph[su];
      const float old = c.lab[src][su];
      const float nl = updated_label(tw, tl, old, e.fast_div);
      c.lab[src ^ 1][su] = nl;
      c.flags[su] |= 3;
      changed = fabsf(nl - old) > e.delta;
      ++c.visits[su];  // a slot is in a list at most once
      c.lastpass[g] = k;
      if (rec_any) {
        const GraphRec &r = e.recs[g];
        const int kg = k + r.ba.pass0;
        if (r.ba.record && kg < kRecordIters) atomicAdd(&r.st.rec_fsizes[kg], 1);
      }
    }
    changed = __shfl_sync(0xffffffffu, changed, 0, G);
    // changed vertex: non-deleted, non-GT neighbours and itself
    // (src/iterativePropagation.cu:200-216). All marks first, then one
    // reservation in the next list for the whole warp.
    unsigned fresh = 0;
    if (changed) {
#pragma unroll
      for (int r = 0; r < R + 1; ++r) {
        const int ns = r < R ? vv[r] : ((gl == 0 && valid) ? su : -1);
        if (ns >= 0 && atomicMax(&c.mark[ns], k + 1) < k + 1) fresh |= 1u << r;
      }
    }
    int add = 0, wide = 0;
#pragma unroll
    for (int r = 0; r < R + 1; ++r)
      if ((fresh >> r) & 1u) {
        const int ns = r < R ? vv[r] : su;
        const int l = c.len[ns];
        if (l == kWideLen) wide = 1;
        else if (c.row[ns] == kNoRow) add += l;
      }
    add = __reduce_add_sync(0xffffffffu, add);
    wide = __reduce_or_sync(0xffffffffu, wide);
    // one reservation in the next list for the whole warp, by a scan of the
    // per-lane counts
    const int nf = __popc(fresh);
    int incl = nf;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    const int tot = __shfl_sync(0xffffffffu, incl, 31);
    int at = 0;
    if (lane == 31 && tot) {
      at = atomicAdd(&c.cnt[nq], tot);
      if (add) atomicAdd(&c.need[nq], add);
      if (wide) c.wide[nq] = 1;
    }
    at = __shfl_sync(0xffffffffu, at, 31) + incl - nf;
#pragma unroll
    for (int r = 0; r < R + 1; ++r)
      if ((fresh >> r) & 1u) next[at++] = static_cast<unsigned short>(r < R ? vv[r] : su);
  }
}

// Team mode of the one-block passes: a small frontier whose rows are all in
// the row pool is run by the block's first kTeamWarps warps, with a named
// barrier (id 1) of those warps between passes, while the other warps of the
// block wait at the block barrier that ends the team stint. The passes and
// their arithmetic are those of the whole block; only fewer warps share the
// rows, and the waiting warps take no issue slots from them.
constexpr int kTeamWarps = 16;
constexpr int kTeamRows = kTeamWarps * 32 / 4;  // rows one round of 4-lane groups takes (8 lanes up to 64)

__device__ __forceinline__ void team_barrier() {
  asm volatile("bar.sync 1, %0;" ::"r"(kTeamWarps * 32) : "memory");
}

// Runs team passes from pass k (stint pass j = k - k0) while the frontier
// stays small and loaded; returns the first pass not run. Called by the
// threads of the first kTeamWarps warps only; every exit decision reads values
// written before the last team barrier, so all of them leave together.
__device__ int team_passes(const EngineArgs &e, SoloCache &c, int k0, int k, int max_iter, bool rec_any,
                           uint64_t t0) {
  const int tid = threadIdx.x;
  const int ng = e.ng;
  // The vertex table and the row pool do not grow during a team stint (it
  // runs only while no row is left to load), so their limits are checked once.
  if (c.used > kVTUse || c.rp_top > kRP) return k;
  // the last pass any limit allows, and the list indices, kept incrementally
  int last = min(max_iter, k0 + kSoloMaxPasses);
  if (e.pass_budget > 0) last = min(last, e.pass_budget);
  const unsigned long long t_launch = e.slice_ns ? ld_relaxed_u64(&e.ectl->t_launch) : 0;
  int q = (k - k0) % 3;
  for (;; ++k) {
    const int j = k - k0;
    const int nq = q == 2 ? 0 : q + 1, z = nq == 2 ? 0 : nq + 1, p = j & 1;
    // every exit condition from values read together (no chain of
    // short-circuit loads)
    const int cnt = c.cnt[q], need = c.need[q], wide = c.wide[q], stop_at = c.stop_at;
    if ((cnt == 0) | (cnt > kTeamRows) | (need > 0) | (wide != 0) | (k >= last) | (j >= stop_at)) break;
    if (tid == 0) {
      c.cnt[z] = 0;
      c.need[z] = 0;
      c.wide[z] = 0;
    }
    if (rec_any)
      for (int g = tid; g < ng; g += kTeamWarps * 32) {
        const GraphRec &r = e.recs[g];
        const int kg = k + 1 + r.ba.pass0;
        if (r.ba.record && kg < kRecordIters) r.st.rec_fsizes[kg] = 0;
      }
    const unsigned short *cur = c.list[p];
    unsigned short *next = c.list[p ^ 1];
    if (cnt <= kTeamWarps * 4) solo_rows<8, kTeamWarps>(e, c, cur, next, cnt, nq, k, rec_any);
    else solo_rows<4, kTeamWarps>(e, c, cur, next, cnt, nq, k, rec_any);
    if (tid == 0 && (j & 15) == 15) {
      const uint64_t now = global_timer_ns();
      if (now - t0 > kSoloBudgetNs) c.stop_at = j + 1;
      if (e.slice_ns != 0 && now - t_launch > e.slice_ns) {  // slice_over without re-reading t_launch
        c.stop_at = j + 1;
        c.stop_slice = 1;
      }
    }
    team_barrier();
    q = nq;
  }
  return k;
}
template <int G>
__device__ void solo_passes(const EngineArgs &e, int k0, int slot, SoloCache &c) {
  const int ng = e.ng;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int kWarps = kBlock / 32;
  constexpr int GPW = 32 / G;
  const int grp = lane / G, gl = lane & (G - 1);
  for (int i = tid; i < kVT; i += kBlock) c.key[i] = kEmptyKey;
  for (int g = tid; g < ng; g += kBlock) c.lastpass[g] = -1;
  if (tid < 3) {
    c.cnt[tid] = 0;
    c.need[tid] = 0;
    c.wide[tid] = 0;
  }
  if (tid == 0) {
    c.used = 0;
    c.rp_top = 0;
    c.stop_at = 0x7fffffff;
    c.stop_slice = 0;
  }
  __syncthreads();
  int max_iter = 0x7fffffff;
  for (int g = 0; g < ng; ++g) max_iter = min(max_iter, e.recs[g].ba.max_iter - e.recs[g].ba.pass0);
  // F_k0 of every graph into the table and list 0
  for (int g = warp; g < ng; g += kWarps) {
    const GraphRec &r = e.recs[g];
    int nn, nw;
    if (!graph_in_pass(r, k0, nn, nw)) continue;
    const int *gl_list = r.st.flist + static_cast<size_t>((k0 + r.ba.pass0) % 3) * r.st.n;
    for (int i = lane; i < nn + nw; i += 32) {
      const int v = i < nn ? gl_list[i] : gl_list[r.st.n - 1 - (i - nn)];
      const int sl = vt_slot(c, e, g, v);
      c.list[0][atomicAdd(&c.cnt[0], 1)] = static_cast<unsigned short>(sl);
    }
  }
  int rec = 0;
  for (int g = tid; g < ng; g += kBlock) {  // recorded sizes of the first pass are counted up below
    const GraphRec &r = e.recs[g];
    const int kg = k0 + r.ba.pass0;
    rec |= r.ba.record;
    if (r.ba.record && kg < kRecordIters) r.st.rec_fsizes[kg] = 0;
  }
  const bool rec_any = __syncthreads_or(rec) != 0;
  {
    int need = 0, wide = 0;
    for (int i = tid; i < c.cnt[0]; i += kBlock) {
      const int su = c.list[0][i];
      if (c.len[su] == kWideLen) wide = 1;
      else need += c.len[su];
    }
    need = __reduce_add_sync(0xffffffffu, need);
    wide = __any_sync(0xffffffffu, wide);
    if (lane == 0) {
      if (need) atomicAdd(&c.need[0], need);
      if (wide) c.wide[0] = 1;
    }
  }
  __syncthreads();
  const uint64_t t0 = global_timer_ns();
  int k = k0;
  int team_from = (e.solo & 4) ? k0 : 0x7fffffff;  // team mode is not tried before this pass
  unsigned long long team_count = 0;  // thread 0: team passes of this stint
  for (;; ++k) {
    const int j = k - k0;
    const int q = j % 3, nq = (j + 1) % 3, p = j & 1;
    const int cnt = c.cnt[q], need = c.need[q], wide = c.wide[q], stop_at = c.stop_at, used = c.used,
              rp_top = c.rp_top;
    // the same decision in every thread: its inputs were last written before
    // the previous barrier (all read together, no chain of short-circuit loads)
    if ((cnt == 0) | (cnt > kSoloList) | (k >= max_iter) | (wide != 0) | (j >= kSoloMaxPasses) | (j >= stop_at) |
        ((e.pass_budget > 0) & (k >= e.pass_budget)) | (used + need > kVTUse) | (rp_top + need > kRP))
      break;
    if (need == 0 && cnt <= kTeamRows && k >= team_from) {
      if (warp < kTeamWarps) {
        const int kk = team_passes(e, c, k0, k, max_iter, rec_any, t0);
        if (tid == 0) c.team_end = kk;
      }
      __syncthreads();  // the other warps wait here for the whole team stint
      const int kk = c.team_end;
      if (tid == 0) team_count += kk - k;
      if (kk == k) team_from = k + 1;  // no pass taken: the block runs this one
      k = kk - 1;  // the loop increment resumes at pass kk
      continue;
    }
    if (need > 0) {
      __syncthreads();  // every thread has read used / rp_top above
      // load the rows of frontier vertices seen for the first time
      for (int base = warp * GPW; base < cnt; base += kWarps * GPW) {
        const int item = base + grp;
        int su = 0, len = 0;
        bool load = false;
        if (item < cnt) {
          su = c.list[p][item];
          load = c.row[su] == kNoRow;
          len = c.len[su];
        }
        int off = 0;
        if (load && gl == 0) off = atomicAdd(&c.rp_top, len);
        off = __shfl_sync(0xffffffffu, off, lane & ~(G - 1));
        if (load) {
          const int g = c.graph[su];
          const DevState &s = e.recs[g].st;
          const int rs = s.full_row[static_cast<int>(c.key[su] & 0xffffffffu)];
          for (int ee = gl; ee < len; ee += G) {
            const int2 ent = s.act_adj[rs + ee];
            const int ns = ent.x >= 0 ? vt_slot(c, e, g, ent.x) : -1;
            c.rp[off + ee] = make_int2(ns, ent.y);
          }
          if (gl == 0) c.row[su] = static_cast<unsigned short>(off);
        }
      }
      __syncthreads();
    }
    // counters of the list filled next pass, and recorded sizes of the next pass
    if (tid == 0) {
      const int z = (j + 2) % 3;
      c.cnt[z] = 0;
      c.need[z] = 0;
      c.wide[z] = 0;
    }
    if (rec_any)
      for (int g = tid; g < ng; g += kBlock) {
        const GraphRec &r = e.recs[g];
        const int kg = k + 1 + r.ba.pass0;
        if (r.ba.record && kg < kRecordIters) r.st.rec_fsizes[kg] = 0;
      }
    // the pass: every frontier row from shared memory, with the widest lane
    // groups that still take the whole frontier in one round of the block
    // (8 lanes up to 64 rows, 4 up to 128, else 2)
    const unsigned short *cur = c.list[p];
    unsigned short *next = c.list[p ^ 1];
    if (cnt <= kBlock / 8) solo_rows<8, kWarps>(e, c, cur, next, cnt, nq, k, rec_any);
    else if (cnt <= kBlock / 4) solo_rows<4, kWarps>(e, c, cur, next, cnt, nq, k, rec_any);
    else solo_rows<2, kWarps>(e, c, cur, next, cnt, nq, k, rec_any);
    // time budgets: checked by thread 0, they stop the stint two passes on
    // (a thread still at the top of this pass must not see the request)
    if (tid == 0 && (j & 15) == 15) {
      if (global_timer_ns() - t0 > kSoloBudgetNs) c.stop_at = j + 1;
      if (slice_over(e)) {
        c.stop_at = j + 1;
        c.stop_slice = 1;
      }
    }
    __syncthreads();
  }
  if (tid == 0 && c.stop_slice) e.ectl->slice_stop = stop_code(e, k);  // the grid resumes at pass k and stops
  const int jq = (k - k0) % 3, jp = (k - k0) & 1;
  // labels written during the stint go back to HBM, with the visit counts
  for (int i = tid; i < kVT; i += kBlock) {
    if (c.key[i] == kEmptyKey) continue;
    const DevState &s = e.recs[c.graph[i]].st;
    const int vis = c.visits[i];
    if (vis) {
      atomicAdd(&s.bc->aff_edges, static_cast<unsigned long long>(vis) * c.len[i]);
      atomicAdd(&s.bc->front_visits, static_cast<unsigned long long>(vis));
    }
    if (!(c.flags[i] & 1)) continue;
    const int v = static_cast<int>(c.key[i] & 0xffffffffu);
    s.lab0[v] = c.lab[0][i];
    s.lab1[v] = c.lab[1][i];
  }
  // per-graph pass counts, and the frontier back into the set of the graph's
  // pass k + pass0 (the set after it empty)
  for (int g = tid; g < ng; g += kBlock) {
    BatchCounters *bc = e.recs[g].st.bc;
    const int kg = k + e.recs[g].ba.pass0;
    if (c.lastpass[g] >= 0) bc->passes = c.lastpass[g] + e.recs[g].ba.pass0 + 1;
    bc->front_count[kg % 3][0] = bc->front_count[kg % 3][1] = 0;
    bc->front_count[(kg + 1) % 3][0] = bc->front_count[(kg + 1) % 3][1] = 0;
  }
  __syncthreads();
  const int cnt = c.cnt[jq];
  for (int i = tid; i < cnt; i += kBlock) {
    const int su = c.list[jp][i];
    const GraphRec &r = e.recs[c.graph[su]];
    const DevState &s = r.st;
    const int v = static_cast<int>(c.key[su] & 0xffffffffu);
    const int set = (k + r.ba.pass0) % 3;
    int *list = s.flist + static_cast<size_t>(set) * s.n;
    if (c.len[su] == kWideLen) list[s.n - 1 - atomicAdd(&s.bc->front_count[set][1], 1)] = v;
    else list[atomicAdd(&s.bc->front_count[set][0], 1)] = v;
  }
  // vertices that were in a frontier join the touched list the first time in
  // this batch; their stamp is the graph's own last pass (below the next grid
  // pass's stamp of a running graph and below the next batch's first stamp)
  for (int i = tid; i < kVT; i += kBlock) {
    if (c.key[i] == kEmptyKey || !(c.flags[i] & 2)) continue;
    const GraphRec &r = e.recs[c.graph[i]];
    const DevState &s = r.st;
    const int v = static_cast<int>(c.key[i] & 0xffffffffu);
    const unsigned g0 = s.ctl->stamp_base + 1u;
    const unsigned old = atomicMax(&s.front_stamp[v], g0 + static_cast<unsigned>(s.bc->passes));
    if (old < g0) {
      const int q = r.ba.seq & 1;
      s.touched[static_cast<size_t>(q) * s.n + atomicAdd(&s.ctl->touched_count[q], 1)] = v;
    }
  }
  if (tid == 0) {
    e.ectl->solo_k[slot] = k;
    e.ectl->solo_passes[slot] = k - k0;
    e.ectl->mode_passes[1] += team_count;  // their time is part of the one-block stint's
  }
}

// One row of at most kLaneRow live entries by one lane, its 8-slot tree in
// registers (slot t = entry t). For such a row the reference's tree over 256
// slots adds only +0 at strides 128..8, so strides 4, 2, 1 give exactly its
// sum — the same as narrow_row<G>. cand[] and wide_bits as in narrow_row.
constexpr int kLaneRow = 8;

__device__ __forceinline__ void lane_row(const DevState &s, const float *src, float *dst, float delta, bool fast,
                                         int u, int rs, int len, bool valid, int (&cand)[kLaneRow + 1],
                                         unsigned &wide_bits) {
  float sw[kLaneRow], sl[kLaneRow];
  int vv[kLaneRow];
  unsigned wb = 0;
  const float old = valid ? src[u] : 0.0f;
#pragma unroll
  for (int t = 0; t < kLaneRow; ++t) {
    sw[t] = 0.0f;
    sl[t] = 0.0f;
    vv[t] = -1;
    if (valid && t < len) {
      const int2 ent = s.act_adj[rs + t];
      if (ent.x >= 0) {
        const float wt = __int_as_float(ent.y);
        sw[t] = wt;                               // 0 + w
        sl[t] = __fmaf_rn(wt, src[ent.x], 0.0f);  // fma(w, F_v, 0)
        const unsigned meta = s.nmeta[ent.x];
        if (meta & 1u) vv[t] = ent.x;
        if (meta & 2u) wb |= 1u << t;
      }
    }
  }
#pragma unroll
  for (int h = kLaneRow / 2; h >= 1; h >>= 1)
#pragma unroll
    for (int t = 0; t < h; ++t) {
      sw[t] = sw[t] + sw[t + h];
      sl[t] = sl[t] + sl[t + h];
    }
  bool changed = false;
  if (valid) {
    const float nl = updated_label(sw[0], sl[0], old, fast);
    dst[u] = nl;
    changed = fabsf(nl - old) > delta;
  }
#pragma unroll
  for (int t = 0; t < kLaneRow; ++t) cand[t] = changed ? vv[t] : -1;
  cand[kLaneRow] = changed ? u : -1;
  wide_bits = changed ? wb : 0u;
}

// Marks of one-lane rows: every stamp atomic is issued before any result is
// used; then the lanes of one graph (a contiguous run: the work list is
// sorted by graph, invalid lanes last) reserve their next-frontier and
// touched-list entries with one atomic per list per run.
__device__ __forceinline__ void lane_mark(const GV &w, bool valid, int key, const int (&cand)[kLaneRow + 1],
                                          unsigned wide_bits, unsigned stamp, int set, int lane) {
  constexpr int C = kLaneRow + 1;
  const DevState &s = w.s;
  unsigned old[C];
#pragma unroll
  for (int r = 0; r < C; ++r) old[r] = cand[r] >= 0 ? atomicMax(&s.front_stamp[cand[r]], stamp) : stamp;
  int nn = 0, nw = 0, nf = 0;
#pragma unroll
  for (int r = 0; r < C; ++r) {
    if (old[r] < stamp) {
      if ((wide_bits >> r) & 1u) ++nw;
      else ++nn;
    }
    if (old[r] < w.g0) ++nf;
  }
  // counts packed 10 bits each (a run of 32 lanes marks at most 288)
  const int mine = nn | (nw << 10) | (nf << 20);
  int incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    const int kp = __shfl_up_sync(0xffffffffu, key, o);
    if (lane >= o && kp == key) incl += t;
  }
  const unsigned peers = __match_any_sync(0xffffffffu, key);
  const int tail = 31 - __clz(peers);
  const int tot = __shfl_sync(0xffffffffu, incl, tail);
  int bn = 0, bw = 0, bf = 0;
  // the run's last lane reserves for the whole run, whether or not it marked
  // anything itself (its own row may be one for the 4-lane groups)
  if (lane == tail && tot != 0) {
    const int tn = tot & 1023, tw = (tot >> 10) & 1023, tf = tot >> 20;
    if (tn) bn = atomicAdd(&s.bc->front_count[set][0], tn);
    if (tw) bw = atomicAdd(&s.bc->front_count[set][1], tw);
    if (tf) bf = atomicAdd(&s.ctl->touched_count[w.a.seq & 1], tf);
  }
  bn = __shfl_sync(0xffffffffu, bn, tail);
  bw = __shfl_sync(0xffffffffu, bw, tail);
  bf = __shfl_sync(0xffffffffu, bf, tail);
  if (!valid || mine == 0) return;
  const int excl = incl - mine;
  int on = bn + (excl & 1023), ow = bw + ((excl >> 10) & 1023), of = bf + (excl >> 20);
  int *list = s.flist + static_cast<size_t>(set) * s.n;
  int *touched = s.touched + static_cast<size_t>(w.a.seq & 1) * s.n;
#pragma unroll
  for (int r = 0; r < C; ++r) {
    if (old[r] < stamp) {
      if ((wide_bits >> r) & 1u) list[s.n - 1 - ow++] = cand[r];
      else list[on++] = cand[r];
    }
    if (old[r] < w.g0) touched[of++] = cand[r];
  }
}

// One propagation pass k over the flattened frontier, by the warps
// [warp0, warp0 + nwarps) and threads [t0, t0 + nthreads) of the launch.
template <int G>
__device__ void run_pass(const EngineArgs &e, int k, const int *pref, int tn, const int *pref2, int tw, int lane,
                         int warp0, int nwarps, int t0, int nthreads) {
  const int ng = e.ng;
  constexpr int GPW = 32 / G;
  const int grp = lane / G, gl = lane & (G - 1);
  // per graph: the set filled two passes from now was last read one pass ago
  for (int g = t0; g < ng; g += nthreads) {
    const GraphRec &r = e.recs[g];
    const int kg = k + r.ba.pass0;
    int nn, nw;
    const bool in = graph_in_pass(r, k, nn, nw);
    r.st.bc->front_count[(kg + 2) % 3][0] = 0;
    r.st.bc->front_count[(kg + 2) % 3][1] = 0;
    if (in) {
      r.st.bc->passes = kg + 1;
      if (r.ba.record && kg < kRecordIters) r.st.rec_fsizes[kg] = nn + nw;
    }
  }
  // A frontier large enough to give every warp two or more rounds of G-lane
  // groups runs with one lane per short row instead: 32 rows in flight per
  // warp rather than 32 / G, so a warp's dependent memory round trips overlap
  // across four to eight times more rows. Smaller frontiers keep the groups,
  // which spread one row's entries over G lanes. Same results either way.
  const bool lane_rows = G == 1 || tn >= 2 * nwarps * GPW;
  if (lane_rows) {
    // rows of at most 32 entries: one lane per row of at most 8 entries, 32
    // rows in flight per warp; rows of 9 to 32 entries of the same 32 go to
    // 4-lane groups afterwards
    // A lane's row of the next round is looked up while this round's rows
    // are in flight: its frontier entry is loaded at the top of the round,
    // its row start and length once this round's gathers are done. The
    // frontier list and the row table do not change during a pass.
    const int stride = nwarps * 32;
    auto entry_of = [&](int item, int &g, int &u) {
      g = 0;
      u = 0;
      if (item < tn) {
        g = locate(pref, ng, item);
        const GraphRec &r = e.recs[g];
        u = r.st.flist[static_cast<size_t>((k + r.ba.pass0) % 3) * r.st.n + (item - pref[g])];
      }
    };
    int g, u, rs = 0, len = 0;
    entry_of(warp0 * 32 + lane, g, u);
    if (warp0 * 32 + lane < tn) {
      const int2 ri = e.recs[g].st.rowinfo[u];
      rs = ri.x;
      len = ri.y;
    }
    for (int base = warp0 * 32; base < tn; base += stride) {
      const int item = base + lane;
      const bool valid = item < tn;
      int g1, u1, rs1 = 0, len1 = 0;
      entry_of(item + stride, g1, u1);
      {
        const GV w = view(e, g);
        const DevState &s = w.s;
        const int kg = k + w.a.pass0;
        const int cb = s.ctl->cur_buf;
        const float *src = ((cb ^ kg) & 1) ? s.lab1 : s.lab0;
        float *dst = ((cb ^ kg) & 1) ? s.lab0 : s.lab1;
        const bool mine = valid && len <= kLaneRow;
        int cand[kLaneRow + 1];
        unsigned wide_bits = 0;
        lane_row(s, src, dst, w.a.delta, e.fast_div, u, rs, len, mine, cand, wide_bits);
        if (item + stride < tn) {
          const int2 ri = e.recs[g1].st.rowinfo[u1];
          rs1 = ri.x;
          len1 = ri.y;
        }
        lane_mark(w, mine, valid ? g : -1, cand, wide_bits, w.g0 + static_cast<unsigned>(kg) + 1u, (kg + 1) % 3,
                  lane);
        add_keyed(mine, static_cast<unsigned>(len), &s.bc->aff_edges);
        add_keyed(mine, 1u, &s.bc->front_visits);
        // the 4-lane groups below take this round's long rows
        const int gc = g, uc = u, lc = len;
        g = g1;
        u = u1;
        rs = rs1;
        len = len1;
        g1 = gc;
        u1 = uc;
        len1 = lc;
      }
      unsigned longm = __ballot_sync(0xffffffffu, valid && len1 > kLaneRow);
      const int q = lane >> 2, ql = lane & 3;
      while (longm) {  // up to 8 rows a round, the q-th remaining one to 4-lane group q
        unsigned m = longm;
        for (int i = 0; i < q && m; ++i) m &= m - 1;
        const bool have = m != 0;
        const int from = have ? __ffs(m) - 1 : 0;
        const int gq = __shfl_sync(0xffffffffu, g1, from);
        const int uq = __shfl_sync(0xffffffffu, u1, from);
        for (int i = 0; i < 8 && longm; ++i) longm &= longm - 1;
        const GV w = view(e, gq);
        const DevState &s = w.s;
        const int kg = k + w.a.pass0;
        const int cb = s.ctl->cur_buf;
        const float *src = ((cb ^ kg) & 1) ? s.lab1 : s.lab0;
        float *dst = ((cb ^ kg) & 1) ? s.lab0 : s.lab1;
        int lq = 0;
        int cand[32 / 4 + 1];
        unsigned wide_bits = 0;
        narrow_row<4>(s, src, dst, w.a.delta, e.fast_div, uq, have, ql, lq, cand, wide_bits);
        group_mark<4>(w, cand, wide_bits, w.g0 + static_cast<unsigned>(kg) + 1u, (kg + 1) % 3, ql);
        add_keyed(have && ql == 0, static_cast<unsigned>(lq), &s.bc->aff_edges);
        add_keyed(have && ql == 0, 1u, &s.bc->front_visits);
      }
    }
  } else
  // rows of at most 32 entries: groups of G lanes
  for (int base = warp0 * GPW; base < tn; base += nwarps * GPW) {
    const int item = base + grp;
    const bool valid = item < tn;
    const int g = valid ? locate(pref, ng, item) : 0;
    const GV w = view(e, g);
    const DevState &s = w.s;
    const int kg = k + w.a.pass0;
    const int nset = (kg + 1) % 3;
    const int cb = s.ctl->cur_buf;
    const float *src = ((cb ^ kg) & 1) ? s.lab1 : s.lab0;
    float *dst = ((cb ^ kg) & 1) ? s.lab0 : s.lab1;
    const unsigned stamp = w.g0 + static_cast<unsigned>(kg) + 1u;
    const int u = valid ? s.flist[static_cast<size_t>(kg % 3) * s.n + (item - pref[g])] : 0;
    int len = 0;
    int cand[32 / G + 1];
    unsigned wide_bits = 0;
    narrow_row<G>(s, src, dst, w.a.delta, e.fast_div, u, valid, gl, len, cand, wide_bits);
    group_mark<G>(w, cand, wide_bits, stamp, nset, gl);
    add_keyed(valid && gl == 0, static_cast<unsigned>(len), &s.bc->aff_edges);
    add_keyed(valid && gl == 0, 1u, &s.bc->front_visits);
  }
  // longer rows: one warp each
  for (int wi = warp0; wi < tw; wi += nwarps) {
    const int g = locate(pref2, ng, wi);
    const GV w = view(e, g);
    const DevState &s = w.s;
    const int kg = k + w.a.pass0;
    const int nset = (kg + 1) % 3;
    const int cb = s.ctl->cur_buf;
    const float *src = ((cb ^ kg) & 1) ? s.lab1 : s.lab0;
    float *dst = ((cb ^ kg) & 1) ? s.lab0 : s.lab1;
    const unsigned stamp = w.g0 + static_cast<unsigned>(kg) + 1u;
    const int u = s.flist[static_cast<size_t>(kg % 3) * s.n + (s.n - 1 - (wi - pref2[g]))];
    auto mark = [&](bool cand, int v) {
      bool fresh = false, first = false;
      if (cand) {
        const unsigned old = atomicMax(&s.front_stamp[v], stamp);
        fresh = old < stamp;
        first = old < w.g0;
      }
      frontier_append(w, fresh, first, v, nset);
    };
    wide_row(s, src, dst, w.a.delta, e.fast_div, u, lane, mark);
    if (lane == 0) {
      atomicAdd(&s.bc->aff_edges, static_cast<unsigned long long>(s.act_len[u]));
      atomicAdd(&s.bc->front_visits, 1ull);
    }
  }
}

// Frontier sizes of pass k: narrow rows into pref, wide rows into pref2. Both
// prefixes come from one scan: a graph's two counts are read once and summed
// as the halves of one 64-bit value (a frontier never reaches 2^32 rows).
__device__ __forceinline__ void pass_sizes(const EngineArgs &e, int k, int *pref, int *pref2, int &tn, int &tw) {
  __shared__ unsigned long long s_warp2[kBlock / 32];
  const int ng = e.ng;
  __syncthreads();
  constexpr int kPer = (kMaxGraphs + kBlock - 1) / kBlock;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long vals[kPer];
  unsigned long long local = 0;
  const int start = threadIdx.x * kPer;
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    const int g = start + j;
    int nn = 0, nw = 0;
    if (g < ng && !graph_in_pass(e.recs[g], k, nn, nw)) nn = nw = 0;
    vals[j] = (static_cast<unsigned long long>(nw) << 32) | static_cast<unsigned>(nn);
    local += vals[j];
  }
  unsigned long long incl = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_warp2[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    unsigned long long x = lane < kBlock / 32 ? s_warp2[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane < kBlock / 32) s_warp2[lane] = x;
  }
  __syncthreads();
  unsigned long long run = incl - local + (warp > 0 ? s_warp2[warp - 1] : 0);
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    const int g = start + j;
    if (g < ng) {
      pref[g] = static_cast<int>(run & 0xffffffffu);
      pref2[g] = static_cast<int>(run >> 32);
    }
    run += vals[j];
  }
  if (threadIdx.x == kBlock - 1) {
    pref[ng] = static_cast<int>(run & 0xffffffffu);
    pref2[ng] = static_cast<int>(run >> 32);
  }
  __syncthreads();
  tn = pref[ng];
  tw = pref2[ng];
}

// Sub-grid mode: mid-size frontiers are run by the first kSubBlocks blocks
// with their own (cheaper) barrier while the other blocks wait at the next
// grid barrier; the passes are those of the full grid.
constexpr int kSubBlocks = 16;
static_assert(kSubEntryMax <= kSubLive, "the sub-grid mode leaves above kSubLive");

template <int G>
__device__ bool sub_passes(const EngineArgs &e, int k0, int slot, int solo_from, int *pref, int *pref2) {
  const int lane = threadIdx.x & 31;
  const int warp0 = blockIdx.x * (kBlock / 32), nwarps = kSubBlocks * (kBlock / 32);
  const int t0 = blockIdx.x * kBlock + threadIdx.x, nthreads = kSubBlocks * kBlock;
  const uint64_t start = global_timer_ns();
  int k = k0;
  for (;; ++k) {
    int tn, tw;
    pass_sizes(e, k, pref, pref2, tn, tw);
    const bool stop = ld_relaxed_u64(&e.ectl->sub_stop) == stop_code(e, k);
    if (tn + tw == 0 || tn + tw > kSubLive || stop || (e.pass_budget > 0 && k >= e.pass_budget)) break;
    // a frontier the one-block mode can take goes back to it (cheaper passes),
    // unless that mode recently could not hold its working set
    if (k > k0 && (e.solo & 1) && tn + tw <= e.solo_entry && k >= solo_from) break;
    run_pass<G>(e, k, pref, tn, pref2, tw, lane, warp0 + (threadIdx.x >> 5), nwarps, t0, nthreads);
    if (t0 == 0 && ((k - k0) & 31) == 31 && global_timer_ns() - start > 100000000ull)
      e.ectl->sub_stop = stop_code(e, k + 1);
    if (t0 == 0 && ((k - k0) & 7) == 7 && slice_over(e)) {
      e.ectl->sub_stop = stop_code(e, k + 1);
      e.ectl->slice_stop = stop_code(e, k + 1);
    }
    if (!grid_sync_n(&e.ectl->sub_bar, kSubBlocks, &e.ectl->err, e.timeout_ns)) return false;
  }
  if (t0 == 0) {
    e.ectl->solo_k[slot] = k;
    e.ectl->solo_passes[slot] = k - k0;
  }
  return true;
}

// The propagation passes of the launch; k_end is the first pass not run (the
// graphs whose frontier is live at k_end continue in a later launch).
template <int G>
__device__ bool phase_g(const EngineArgs &e, const Ctx &c, int *pref, int *pref2, SoloCache &solo, int &k_end) {
  int no_small_at = -1;  // a pass the small modes declined goes to the full grid
  int solo_from = 0;     // the one-block mode declined: not tried again before this pass
  int stint = 0;
  int k = 0;
  // thread 0 of block 0: passes and device time per mode in this launch
  unsigned long long mp[3] = {0, 0, 0}, mns[3] = {0, 0, 0};  // one block, sub-grid, full grid
  for (;; ++k) {
    int tn, tw;
    pass_sizes(e, k, pref, pref2, tn, tw);
    if (tn + tw == 0) break;
    if (e.pass_budget > 0 && k >= e.pass_budget) break;
    if (ld_relaxed_u64(&e.ectl->slice_stop) == stop_code(e, k)) break;
    if (c.gtid == 0) e.ectl->where_pass = k;
    const bool solo_ok = (e.solo & 1) && tn + tw <= e.solo_entry && k != no_small_at && k >= solo_from;
    const bool sub_ok = !solo_ok && (e.solo & 2) && gridDim.x > 2 * kSubBlocks && tn + tw <= e.sub_entry &&
                        k != no_small_at;
    if (solo_ok || sub_ok) {
      const uint64_t ts = c.gtid == 0 ? global_timer_ns() : 0;
      if (solo_ok) {
        if (blockIdx.x == 0) solo_passes<kSoloG>(e, k, stint & 1, solo);
      } else if (blockIdx.x < kSubBlocks) {
        if (!sub_passes<G>(e, k, stint & 1, solo_from, pref, pref2)) return false;
      }
      if (!grid_sync(&e.ectl->bar, &e.ectl->err, e.timeout_ns)) return false;
      const int done = ld_relaxed_i32(&e.ectl->solo_passes[stint & 1]);
      const int kk = ld_relaxed_i32(&e.ectl->solo_k[stint & 1]);
      ++stint;
      if (c.gtid == 0) {
        mp[solo_ok ? 0 : 1] += done;
        mns[solo_ok ? 0 : 1] += global_timer_ns() - ts;
      }
      if (done == 0) no_small_at = k;
      if (solo_ok && done == 0) solo_from = k + 256;
      k = kk - 1;  // the loop increment resumes at pass kk
      continue;
    }
    const uint64_t tp = c.gtid == 0 ? global_timer_ns() : 0;
    run_pass<G>(e, k, pref, tn, pref2, tw, c.lane, c.gwarp, c.nwarps, c.gtid, c.nthreads);
    if (c.gtid == 0 && slice_over(e)) e.ectl->slice_stop = stop_code(e, k + 1);
    if (!grid_sync(&e.ectl->bar, &e.ectl->err, e.timeout_ns)) return false;
    if (c.gtid == 0) {
      ++mp[2];
      mns[2] += global_timer_ns() - tp;
    }
  }
  k_end = k;
  if (c.gtid == 0) {
    e.ectl->mode_passes[0] += mp[0];
    e.ectl->mode_ns[0] += mns[0];
    e.ectl->mode_passes[2] += mp[1];
    e.ectl->mode_ns[2] += mns[1];
    e.ectl->mode_passes[3] += mp[2];
    e.ectl->mode_ns[3] += mns[2];
  }
  return true;
}

// A graph's batch ends in this launch when it takes no part in pass k_end.
__device__ __forceinline__ bool batch_done(const GraphRec &r, int k_end) {
  int nn, nw;
  return !graph_in_pass(r, k_end, nn, nw);
}

// ---------------------------------------------------------------- phase H ---
// Ground truth of this batch back to exactly 0/1 in both buffers
// (src/iterativePropagation.cu:224-235; earlier ground truth already is), and
// the accuracy counters (src/dynLP.cu:65-85) updated at every vertex whose
// status or label may have changed.
__device__ void phase_h(const EngineArgs &e, const Ctx &c, int *pref, int k_end) {
  const int ng = e.ng;
  const int total = flat_build(pref, ng, [&](int g) {
    const GraphRec &r = e.recs[g];
    if (!batch_done(r, k_end)) return 0;
    return r.ba.G + r.ba.D + r.st.ctl->touched_count[r.ba.seq & 1] + r.ba.I + r.ba.D + r.ba.G;
  });
  flat_threads(c, pref, ng, total, [&](int g, int i, bool valid) {
    const GraphRec &r = e.recs[g];
    const DevState &s = r.st;
    const BatchArgs &a = r.ba;
    int dc = 0, dt = 0;
    if (valid) {
      if (i < a.G) {
        const int v = a.gt_ids[i];
        const float l = s.gt[v] == 0 ? 0.0f : 1.0f;
        s.lab0[v] = l;
        s.lab1[v] = l;
      } else if ((i -= a.G) < a.D) {
        s.del_keep[i] = a.del[i];  // the next batch restores these rows (ref)
      } else {
        i -= a.D;
        const int tc = s.ctl->touched_count[a.seq & 1];
        int v;
        if (i < tc) v = s.touched[static_cast<size_t>(a.seq & 1) * s.n + i];
        else if ((i -= tc) < a.I) v = a.ins[i];
        else if ((i -= a.I) < a.D) v = a.del[i];
        else v = a.gt_ids[i - a.D];
        const int st = s.status[v];
        int now = -1;
        if (st != kDeleted && st != kGroundTruth) {
          const int passes = s.bc->passes;
          const float *lab = ((s.ctl->cur_buf ^ passes) & 1) ? s.lab1 : s.lab0;
          const int pred = lab[v] >= 0.5f ? 1 : 0;
          const int truth = s.truth ? s.truth[v] : 0;
          now = pred == truth ? 1 : 0;
        }
        const int before = atomicExch(&s.contrib[v], now);
        dc = (now == 1) - (before == 1);
        dt = (now >= 0) - (before >= 0);
      }
    }
    const unsigned act = __ballot_sync(0xffffffffu, valid && (dc != 0 || dt != 0));
    if (valid && (dc != 0 || dt != 0)) {
      const unsigned peers = __match_any_sync(act, reinterpret_cast<unsigned long long>(s.ctl));
      const int sc = __reduce_add_sync(peers, dc);
      const int st2 = __reduce_add_sync(peers, dt);
      if ((threadIdx.x & 31) == __ffs(peers) - 1) {
        if (sc) atomicAdd(reinterpret_cast<unsigned long long *>(&s.ctl->correct), static_cast<unsigned long long>(static_cast<long long>(sc)));
        if (st2) atomicAdd(reinterpret_cast<unsigned long long *>(&s.ctl->total), static_cast<unsigned long long>(static_cast<long long>(st2)));
      }
    }
  });
}

}  // namespace

template <int G>
__global__ void __launch_bounds__(kBlock, 1024 / kBlock) engine_kernel(EngineArgs e) {
  const Ctx c = make_ctx();
  __shared__ int pref[kMaxGraphs + 1];
  __shared__ int pref2[kMaxGraphs + 1];
  extern __shared__ __align__(16) unsigned char dsmem[];
  SoloCache &solo = *reinterpret_cast<SoloCache *>(dsmem);
  GridBarrier *bar = &e.ectl->bar;
  int *err = &e.ectl->err;
  const uint64_t to = e.timeout_ns;
  if (ld_relaxed_i32(err) != 0) return;

  // block 0 records the last phase it reached (read back after a timeout)
  auto at = [&](int phase) {
    if (blockIdx.x == 0 && threadIdx.x == 0) e.ectl->where = phase;
  };
  if (c.gtid == 0) e.ectl->t_launch = global_timer_ns();
  if (e.ng_new > 0) {  // a launch that only continues batches starts at phase G
    at(1);
    phase_a(e, c, pref);
    if (!grid_sync(bar, err, to)) return;
    at(2);
    phase_b(e, c, pref);
    if (!grid_sync(bar, err, to)) return;
    at(3);
    phase_c(e, c, pref);
    if (!grid_sync(bar, err, to)) return;
    at(4);
    phase_d_frontier(e, c, pref);
    if (!phase_d_sv(e, c, pref)) return;
    at(5);
    if (!grid_sync(bar, err, to)) return;
    at(6);
    phase_e(e, c, pref);
    if (!grid_sync(bar, err, to)) return;
    at(7);
    phase_f(e, c, pref);
    if (!grid_sync(bar, err, to)) return;
  }
  at(8);
  int k_end = 0;
  if (!phase_g<G>(e, c, pref, pref2, solo, k_end)) return;
  at(9);
  phase_h(e, c, pref, k_end);
  if (!grid_sync(bar, err, to)) return;
  at(10);

  // per-graph statistics and the state the next batch starts from
  for (int g = c.gtid; g < e.ng; g += c.nthreads) {
    const GraphRec &r = e.recs[g];
    const DevState &s = r.st;
    const BatchArgs &a = r.ba;
    const BatchCounters *bc = s.bc;
    if (!batch_done(r, k_end)) {  // continues in a later launch
      if (e.progress) e.progress[g] = make_int2(0, k_end + a.pass0);
      continue;
    }
    if (e.progress) e.progress[g] = make_int2(1, bc->passes);
    const GV w = view(e, g);
    const bool comp = w.comp_path();
    const int passes = bc->passes;
    const int hc = hook_count(w);
    int rounds = 0;
    if (hc > 0) {
      rounds = kMaxHookRounds;
      for (int q = 0; q < kMaxHookRounds; ++q)
        if (bc->hook_flag[q] == 0) {
          rounds = q + 1;
          break;
        }
    }
    dlp_batch_stats st;
    memset(&st, 0, sizeof(st));
    st.batch = a.batch;
    st.iterations = passes;
    st.num_components = comp ? bc->num_comp : 0;
    st.num_sub_edges = comp ? 2 * bc->num_kept : 0;
    st.hook_edges = a.spec ? 2 * hc : hc;
    st.hook_rounds = rounds;
    st.seed_frontier = bc->seed_frontier;
    st.seed_marks = bc->num_seeds;
    st.affected_edges = static_cast<int64_t>(bc->aff_edges);
    st.frontier_visits = static_cast<int64_t>(bc->front_visits);
    st.correct = s.ctl->correct;
    st.total = s.ctl->total;
    st.accuracy = st.total > 0 ? static_cast<float>(st.correct) / static_cast<float>(st.total) : 1.0f;
    st.status = DLP_OK;
    st.init_branch = comp ? 1 : (a.I > 0 ? 2 : 0);
    st.hook_truncated = (!a.spec && comp && 2 * bc->num_kept > a.E) ? 1 : 0;
    st.dirty_rows = bc->num_dirty;
    st.dirty_entries = static_cast<int64_t>(bc->dirty_entries);
    *s.stats_slot = st;
    s.ctl->cur_buf ^= (passes & 1);
    s.ctl->stamp_base = w.g0 + static_cast<unsigned>(passes) + 1u;
  }
}

template __global__ void engine_kernel<1>(EngineArgs);
template __global__ void engine_kernel<4>(EngineArgs);
template __global__ void engine_kernel<8>(EngineArgs);
template __global__ void engine_kernel<16>(EngineArgs);
template __global__ void engine_kernel<32>(EngineArgs);

// One block per graph that starts a batch: its counters back to zero.
__global__ void zero_counters_kernel(const GraphRec *recs) {
  int *p = reinterpret_cast<int *>(recs[blockIdx.x].st.bc);
  constexpr int kWords = static_cast<int>(sizeof(BatchCounters) / sizeof(int));
  for (int i = threadIdx.x; i < kWords; i += blockDim.x) p[i] = 0;
}

void launch_zero_counters(const GraphRec *recs, int ng_new, cudaStream_t stream) {
  if (ng_new > 0) zero_counters_kernel<<<ng_new, 128, 0, stream>>>(recs);
}

size_t engine_dynamic_smem() { return sizeof(SoloCache); }

const void *engine_kernel_ptr(int lanes) {
  switch (lanes) {
    case 1: return reinterpret_cast<const void *>(&engine_kernel<1>);
    case 4: return reinterpret_cast<const void *>(&engine_kernel<4>);
    case 8: return reinterpret_cast<const void *>(&engine_kernel<8>);
    case 16: return reinterpret_cast<const void *>(&engine_kernel<16>);
    case 32: return reinterpret_cast<const void *>(&engine_kernel<32>);
    default: return nullptr;
  }
}

}  // namespace engine
}  // namespace dlp
