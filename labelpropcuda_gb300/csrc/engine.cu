// Host side of the batch engine (C ABI groups 2 and 2b in dlp_gb300.h): a set
// of resident graphs, and steps that apply one batch to each of several graphs
// in one cooperative launch. dlp_session is the one-graph engine.
//
// Memory layout in HBM, per resident graph (n vertices, m directed edges):
//   full_row  int32[n+1]     full_adj int2[m] {col, weight bits}
//   act_adj   int2[m]        live rows in the same slots as full_adj
//   act_len   int32[n]       live row length
//   status/gt int8[n]        truth uint8[n]       contrib int32[n]
//   lab0/lab1 fp32[n]        the stale double buffer of the reference
//   stamps    uint32[n] x 4  (deleted, ground truth, dirty, frontier)
//   lists     int32: dirty[n], seeds[n], frontier 3 x [n], touched 2 x [n]
//   SV        par int32[n], acc int64[2n]
//   per batch edge scratch, sized by the largest batch seen
// Nothing is O(n) per batch: every pass walks the batch's lists, the rows next
// to changed vertices, and the frontier.
#include <algorithm>
#include <cstring>
#include <vector>

#include "engine.cuh"

using dlp::engine::EngineArgs;
using dlp::engine::EngineCtl;
using dlp::engine::GraphRec;
using dlp::session::BatchArgs;
using dlp::session::BatchCounters;
using dlp::session::DevState;
using dlp::session::SessionCtl;

namespace {

constexpr int kStepRing = 4096;  // events and statistics kept per graph / per engine

__global__ void interleave_kernel(const int *col, const float *val, int2 *adj, int64_t m) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < m;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    adj[i] = make_int2(col[i], __float_as_int(val[i]));
}

// Every row empty: {row start, 0}.
__global__ void rowinfo_reset_kernel(const int *full_row, int2 *rowinfo, int64_t n) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    rowinfo[i] = make_int2(full_row[i], 0);
}

__global__ void fill_f32_kernel(float *p, float v, int64_t count) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    p[i] = v;
}

size_t align16(size_t x) { return (x + 15) & ~static_cast<size_t>(15); }

int dalloc_bytes(void **p, size_t bytes, std::vector<void *> &owned, size_t &counted,
                 std::vector<size_t> *sizes = nullptr) {
  void *q = nullptr;
  bytes = std::max<size_t>(bytes, 16);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return dlp::fail(e == cudaErrorMemoryAllocation ? DLP_ERR_OUT_OF_MEMORY : DLP_ERR_CUDA,
                     std::string("cudaMalloc of ") + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
  }
  owned.push_back(q);
  if (sizes) sizes->push_back(bytes);
  counted += bytes;
  *p = q;
  return DLP_OK;
}

template <class T>
int dalloc(T **p, size_t count, std::vector<void *> &owned, size_t &counted, std::vector<size_t> *sizes = nullptr) {
  void *q = nullptr;
  DLP_TRY(dalloc_bytes(&q, count * sizeof(T), owned, counted, sizes));
  *p = static_cast<T *>(q);
  return DLP_OK;
}

// Device bytes a resident graph needs (fixed part).
size_t graph_bytes(int64_t n, int64_t m, bool truth, bool bmap, bool record) {
  size_t b = 4 * (n + 1) + 16 * m + 4 * n + 2 * n + 4 * n + 8 * n + 4 * n + 16 * n + 4 * n * 2 + 4 * n * 5 +
             4 * n + 16 * n + n + 8 * n + sizeof(dlp_batch_stats) * kStepRing;
  if (truth) b += n;
  if (bmap) b += 4 * n;
  if (record) b += 4 * n * 4 + 4 * dlp::session::kRecordIters;
  return b;
}

struct GraphSlot {
  int n = 0;
  int64_t m = 0;
  float tau = 0.5f;
  std::vector<void *> owned;
  std::vector<size_t> sizes;  // bytes of each owned array, in allocation order
  bool has_truth = false, has_bmap = false;
  size_t bytes = 0;
  DevState st{};
  dlp_batch_stats *stats = nullptr;  // ring of kStepRing
  // batch scratch (grown)
  int edge_cap = 0, del_cap = 0, keep_cap = 0;
  int *lsrc = nullptr, *ldst = nullptr, *sub_pairs = nullptr, *sub_local = nullptr;
  int *del_pre = nullptr, *del_keep = nullptr;
  // batch bookkeeping
  int seq = 0;
  int prev_d = 0;
  int last_inserted = 0;
  // a batch whose propagation continues in a later sliced step
  bool inflight = false;
  GraphRec inflight_rec{};
  std::vector<int> seq_batch;
  std::vector<int> seq_step;  // engine step of each application

  void free_all() {
    for (void *p : owned) cudaFree(p);
    owned.clear();
    sizes.clear();
    for (void *p : {static_cast<void *>(lsrc), static_cast<void *>(ldst), static_cast<void *>(sub_pairs),
                    static_cast<void *>(sub_local), static_cast<void *>(del_pre), static_cast<void *>(del_keep)})
      cudaFree(p);
    lsrc = ldst = sub_pairs = sub_local = del_pre = del_keep = nullptr;
  }
};

}  // namespace

struct dlp_engine {
  dlp_config cfg{};
  int device = 0;
  int max_graphs = 0;
  size_t budget = 0;
  size_t used = 0;
  int lanes = 8;
  int grid = 0;
  size_t smem = 0;
  const void *kernel = nullptr;
  cudaStream_t stream = nullptr;
  std::vector<void *> owned;
  size_t owned_bytes = 0;
  EngineCtl *ectl = nullptr;
  SessionCtl *ctl_all = nullptr;
  BatchCounters *bc_all = nullptr;
  GraphRec *recs_dev = nullptr;
  GraphRec *recs_host[2] = {nullptr, nullptr};
  cudaEvent_t recs_free[2] = {nullptr, nullptr};
  char *pinned[2] = {nullptr, nullptr};
  size_t pinned_cap[2] = {0, 0};
  cudaEvent_t pinned_free[2] = {nullptr, nullptr};
  char *stage_dev[2] = {nullptr, nullptr};
  size_t stage_cap[2] = {0, 0};
  std::vector<GraphSlot *> graphs;  // by graph id (nullptr: free id)
  std::vector<char> held;           // by graph id: a free id kept for a graph evicted to host memory
  int steps = 0;
  cudaEvent_t ev[kStepRing][2];
  bool ev_made = false;
  int2 *progress_dev = nullptr;     // per launch position: {finished, passes}
  int2 *progress_host = nullptr;    // pinned copy
  int inflight = 0;                 // graphs whose batch continues in a later step
  std::vector<int> last_finished;   // graphs whose batch ended in the last sliced step

  ~dlp_engine() {
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    for (GraphSlot *g : graphs)
      if (g) {
        g->free_all();
        delete g;
      }
    for (void *p : owned) cudaFree(p);
    if (progress_host) cudaFreeHost(progress_host);
    for (int i = 0; i < 2; ++i) {
      if (recs_host[i]) cudaFreeHost(recs_host[i]);
      if (pinned[i]) cudaFreeHost(pinned[i]);
      if (stage_dev[i]) cudaFree(stage_dev[i]);
      if (recs_free[i]) cudaEventDestroy(recs_free[i]);
      if (pinned_free[i]) cudaEventDestroy(pinned_free[i]);
    }
    if (ev_made)
      for (int i = 0; i < kStepRing; ++i) {
        cudaEventDestroy(ev[i][0]);
        cudaEventDestroy(ev[i][1]);
      }
    if (stream) cudaStreamDestroy(stream);
  }
};

struct dlp_session {
  dlp_engine *eng = nullptr;
  int gid = 0;
};

namespace {

GraphSlot *slot_of(dlp_engine *e, int gid) {
  if (!e || gid < 0 || gid >= static_cast<int>(e->graphs.size())) return nullptr;
  return e->graphs[gid];
}

int grow_graph_scratch(dlp_engine *e, GraphSlot *g, int E, int D) {
  if (E > g->edge_cap) {
    int cap = std::max(E, std::max(1024, g->edge_cap * 2));
    cap = (cap + 3) & ~3;
    DLP_CUDA_TRY(cudaStreamSynchronize(e->stream));
    for (int **p : {&g->lsrc, &g->ldst, &g->sub_pairs, &g->sub_local}) {
      cudaFree(*p);
      *p = nullptr;
    }
    g->edge_cap = 0;
    DLP_CUDA_TRY(cudaMalloc(&g->lsrc, sizeof(int) * cap));
    DLP_CUDA_TRY(cudaMalloc(&g->ldst, sizeof(int) * cap));
    DLP_CUDA_TRY(cudaMalloc(&g->sub_pairs, sizeof(int) * 2 * static_cast<size_t>(cap)));
    DLP_CUDA_TRY(cudaMalloc(&g->sub_local, sizeof(int) * 2 * static_cast<size_t>(cap)));
    g->edge_cap = cap;
  }
  if (D > g->del_cap) {
    const int cap = std::max(D, std::max(1024, g->del_cap * 2));
    DLP_CUDA_TRY(cudaStreamSynchronize(e->stream));
    cudaFree(g->del_pre);
    g->del_pre = nullptr;
    g->del_cap = 0;
    DLP_CUDA_TRY(cudaMalloc(&g->del_pre, sizeof(int) * cap));
    g->del_cap = cap;
  }
  if (D > g->keep_cap || !g->del_keep) {
    // keeps the previous batch's deletions (read by the next batch), so the
    // old contents move over
    const int cap = std::max(D, std::max(1024, g->keep_cap * 2));
    int *nk = nullptr;
    DLP_CUDA_TRY(cudaStreamSynchronize(e->stream));
    DLP_CUDA_TRY(cudaMalloc(&nk, sizeof(int) * cap));
    if (g->del_keep && g->prev_d > 0)
      DLP_CUDA_TRY(cudaMemcpy(nk, g->del_keep, sizeof(int) * g->prev_d, cudaMemcpyDeviceToDevice));
    cudaFree(g->del_keep);
    g->del_keep = nk;
    g->keep_cap = cap;
  }
  return DLP_OK;
}

int reset_graph(dlp_engine *e, GraphSlot *g, int gid) {
  const int n = g->n;
  DevState &d = g->st;
  cudaStream_t q = e->stream;
  DLP_CUDA_TRY(cudaStreamSynchronize(q));
  DLP_CUDA_TRY(cudaMemsetAsync(d.act_len, 0, sizeof(int) * n, q));
  DLP_CUDA_TRY(cudaMemsetAsync(d.status, dlp::kDeleted, n, q));
  DLP_CUDA_TRY(cudaMemsetAsync(d.gt, 0xff, n, q));
  DLP_CUDA_TRY(cudaMemsetAsync(d.nmeta, 1, n, q));  // no ground truth, empty rows
  DLP_CUDA_TRY(cudaMemsetAsync(d.contrib, 0xff, sizeof(int) * n, q));
  DLP_CUDA_TRY(cudaMemsetAsync(d.local, 0xff, sizeof(int) * n, q));
  for (unsigned *p : {d.del_stamp, d.gt_stamp, d.dirty_stamp, d.front_stamp})
    DLP_CUDA_TRY(cudaMemsetAsync(p, 0, sizeof(unsigned) * n, q));
  rowinfo_reset_kernel<<<1024, 256, 0, q>>>(d.full_row, d.rowinfo, n);
  fill_f32_kernel<<<1024, 256, 0, q>>>(d.lab0, 0.5f, n);
  fill_f32_kernel<<<1024, 256, 0, q>>>(d.lab1, 0.5f, n);
  DLP_CUDA_TRY(cudaGetLastError());
  DLP_CUDA_TRY(cudaMemsetAsync(e->ctl_all + gid, 0, sizeof(SessionCtl), q));
  DLP_CUDA_TRY(cudaStreamSynchronize(q));
  g->seq = 0;
  g->prev_d = 0;
  g->last_inserted = 0;
  if (g->inflight) {
    g->inflight = false;
    --e->inflight;
  }
  DLP_CUDA_TRY(cudaMemset(e->bc_all + gid, 0, sizeof(BatchCounters)));
  g->seq_batch.clear();
  g->seq_step.clear();
  return DLP_OK;
}

int check_ids(const int *ids, int count, int n, const char *what) {
  if (count < 0) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, std::string("negative count for ") + what);
  if (count > 0 && !ids) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, std::string("null ") + what);
  for (int i = 0; i < count; ++i)
    if (ids[i] < 0 || ids[i] >= n)
      return dlp::fail(DLP_ERR_INVALID_ARGUMENT,
                       std::string("vertex id ") + std::to_string(ids[i]) + " out of range in " + what);
  return DLP_OK;
}

int check_view(const dlp_batch_view *v, int n) {
  if (v->num_inserted < 0 || v->num_gt < 0 || v->num_deleted < 0 || v->num_edges < 0)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "negative batch size");
  if (v->num_inserted > n) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "more inserted entries than vertices");
  if ((v->num_inserted && !v->inserted) || (v->num_gt && (!v->gt_ids || !v->gt_labels)) ||
      (v->num_deleted && !v->deleted) || (v->num_edges && (!v->edge_src || !v->edge_dst || !v->edge_weight)))
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null batch array");
  return DLP_OK;
}

int device_error(dlp_engine *e) {
  int err = 0;
  DLP_CUDA_TRY(cudaMemcpy(&err, &e->ectl->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err != 0)
    return dlp::fail(err, std::string("device reported ") + dlp_status_string(err) +
                              "; the graphs of that step must be reset");
  return DLP_OK;
}

// Options of a sliced launch (continuous batching); the default runs every
// batch of the launch to its end.
struct SliceOpts {
  int pass_budget = 0;
  unsigned long long slice_ns = 0;
  bool resume = false;  // also continue every graph whose batch is unfinished
};

// One launch over `count` graphs that start a batch (device-resident batch
// views), followed, when opts.resume, by every graph whose batch continues.
int launch_step(dlp_engine *e, int count, const int *gids, const int *batch_idx, const dlp_batch_view *dv,
                const SliceOpts &opts = SliceOpts()) {
  std::vector<int> resumed;
  if (opts.resume)
    for (int gid = 0; gid < static_cast<int>(e->graphs.size()); ++gid)
      if (e->graphs[gid] && e->graphs[gid]->inflight) resumed.push_back(gid);
  const int total = count + static_cast<int>(resumed.size());
  if (total <= 0) return DLP_OK;
  if (total > e->max_graphs || total > dlp::engine::kMaxGraphs)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "too many graphs in one step");
  for (int i = 0; i < count; ++i) {
    GraphSlot *g = slot_of(e, gids[i]);
    if (!g) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "unknown graph id");
    if (g->inflight)
      return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "graph " + std::to_string(gids[i]) +
                                                     " has a batch in progress (continue it with a sliced step)");
    for (int j = 0; j < i; ++j)
      if (gids[j] == gids[i]) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "a graph appears twice in one step");
    DLP_TRY(check_view(&dv[i], g->n));
    DLP_TRY(grow_graph_scratch(e, g, dv[i].num_edges, dv[i].num_deleted));
  }
  const int p = e->steps & 1;
  DLP_CUDA_TRY(cudaEventSynchronize(e->recs_free[p]));
  GraphRec *rh = e->recs_host[p];
  const double to = e->cfg.wait_timeout_s > 0 ? e->cfg.wait_timeout_s : 2.0;
  const int slot = e->steps % kStepRing;
  for (int i = 0; i < count; ++i) {
    GraphSlot *g = e->graphs[gids[i]];
    DevState d = g->st;
    d.lsrc = g->lsrc;
    d.ldst = g->ldst;
    d.sub_pairs = g->sub_pairs;
    d.sub_local = g->sub_local;
    d.del_pre = g->del_pre;
    d.del_keep = g->del_keep;
    d.bc = e->bc_all + gids[i];
    d.stats_slot = g->stats + (g->seq % kStepRing);
    BatchArgs a{};
    a.batch = batch_idx[i];
    a.seq = g->seq;
    a.ins = dv[i].inserted;
    a.I = dv[i].num_inserted;
    a.gt_ids = dv[i].gt_ids;
    a.gt_lab = dv[i].gt_labels;
    a.G = dv[i].num_gt;
    a.del = dv[i].deleted;
    a.D = dv[i].num_deleted;
    a.es = dv[i].edge_src;
    a.ed = dv[i].edge_dst;
    a.ew = dv[i].edge_weight;
    a.E = dv[i].num_edges;
    a.prev_del = g->del_keep;
    a.PD = g->prev_d;
    a.tau = g->tau;
    a.delta = e->cfg.delta;
    a.max_iter = e->cfg.max_iterations;
    a.spec = e->cfg.semantics == DLP_SEMANTICS_SPEC;
    a.record = e->cfg.record != 0;
    a.solo = e->cfg.small_frontier_solo != 0;
    a.pass0 = 0;
    a.timeout_ns = static_cast<unsigned long long>(to * 1e9);
    rh[i].st = d;
    rh[i].ba = a;
  }
  for (size_t j = 0; j < resumed.size(); ++j) rh[count + j] = e->graphs[resumed[j]]->inflight_rec;
  GraphRec *recs = e->recs_dev + (p ? e->max_graphs : 0);
  DLP_CUDA_TRY(cudaMemcpyAsync(recs, rh, sizeof(GraphRec) * total, cudaMemcpyHostToDevice, e->stream));
  DLP_CUDA_TRY(cudaEventRecord(e->recs_free[p], e->stream));
  dlp::engine::launch_zero_counters(recs, count, e->stream);
  DLP_CUDA_TRY(cudaGetLastError());
  // every step_sliced call reads back which batches ended, budget or not
  const bool sliced = opts.resume || opts.pass_budget > 0 || opts.slice_ns > 0;
  EngineArgs args{};
  args.recs = recs;
  args.ng = total;
  args.ng_new = count;
  args.ectl = e->ectl;
  args.timeout_ns = static_cast<unsigned long long>(to * 1e9);
  args.solo = e->cfg.small_frontier_solo < 0 ? 7 : e->cfg.small_frontier_solo;
  args.fast_div = e->cfg.arithmetic == DLP_ARITH_REFERENCE_FAST_MATH ? 1 : 0;
  args.solo_entry = e->cfg.solo_entry > 0 ? e->cfg.solo_entry : dlp::engine::kSoloEntryDefault;
  args.sub_entry = e->cfg.subgrid_entry > 0 ? e->cfg.subgrid_entry : dlp::engine::kSubEntryDefault;
  args.pass_budget = opts.pass_budget;
  args.slice_ns = opts.slice_ns;
  args.tag = e->steps + 1;
  args.delta = e->cfg.delta;
  args.progress = sliced ? e->progress_dev : nullptr;
  DLP_CUDA_TRY(cudaEventRecord(e->ev[slot][0], e->stream));
  void *kargs[] = {&args};
  DLP_TRY(dlp::launch_cooperative(e->kernel, e->grid, dlp::session::kBlock, kargs, e->smem, e->stream));
  DLP_CUDA_TRY(cudaEventRecord(e->ev[slot][1], e->stream));
  for (int i = 0; i < count; ++i) {
    GraphSlot *g = e->graphs[gids[i]];
    if (static_cast<int>(g->seq_batch.size()) <= g->seq) {
      g->seq_batch.resize(g->seq + 1);
      g->seq_step.resize(g->seq + 1);
    }
    g->seq_batch[g->seq] = batch_idx[i];
    g->seq_step[g->seq] = e->steps;
    g->prev_d = dv[i].num_deleted;
    g->last_inserted = dv[i].num_inserted;
    ++g->seq;
  }
  ++e->steps;
  if (!sliced) return DLP_OK;
  // which batches ended: the rest continue from their recorded pass
  DLP_CUDA_TRY(cudaMemcpyAsync(e->progress_host, e->progress_dev, sizeof(int2) * total, cudaMemcpyDeviceToHost,
                               e->stream));
  DLP_CUDA_TRY(cudaStreamSynchronize(e->stream));
  DLP_TRY(device_error(e));
  e->last_finished.clear();
  for (int i = 0; i < total; ++i) {
    const int gid = i < count ? gids[i] : resumed[i - count];
    GraphSlot *g = e->graphs[gid];
    const int2 pr = e->progress_host[i];
    const bool was = g->inflight;
    if (pr.x) {
      g->inflight = false;
      e->last_finished.push_back(gid);
    } else {
      g->inflight = true;
      g->inflight_rec = rh[i];
      g->inflight_rec.ba.pass0 = pr.y;
    }
    e->inflight += static_cast<int>(g->inflight) - static_cast<int>(was);
  }
  return DLP_OK;
}

// Host batches of one step -> one pinned buffer -> one H2D copy.
int stage_step(dlp_engine *e, int count, const int *gids, const dlp_batch_view *h, std::vector<dlp_batch_view> &dv) {
  size_t total = 16;
  for (int i = 0; i < count; ++i) {
    GraphSlot *g = slot_of(e, gids[i]);
    if (!g) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "unknown graph id");
    DLP_TRY(check_view(&h[i], g->n));
    DLP_TRY(check_ids(h[i].inserted, h[i].num_inserted, g->n, "inserted"));
    DLP_TRY(check_ids(h[i].gt_ids, h[i].num_gt, g->n, "gt_ids"));
    DLP_TRY(check_ids(h[i].deleted, h[i].num_deleted, g->n, "deleted"));
    DLP_TRY(check_ids(h[i].edge_src, h[i].num_edges, g->n, "edge_src"));
    DLP_TRY(check_ids(h[i].edge_dst, h[i].num_edges, g->n, "edge_dst"));
    total += align16(4 * static_cast<size_t>(h[i].num_inserted)) + 2 * align16(4 * static_cast<size_t>(h[i].num_gt)) +
             align16(4 * static_cast<size_t>(h[i].num_deleted)) + 3 * align16(4 * static_cast<size_t>(h[i].num_edges));
  }
  const int p = e->steps & 1;
  DLP_CUDA_TRY(cudaEventSynchronize(e->pinned_free[p]));
  if (total > e->pinned_cap[p]) {
    if (e->pinned[p]) cudaFreeHost(e->pinned[p]);
    e->pinned[p] = nullptr;
    e->pinned_cap[p] = 0;
    DLP_CUDA_TRY(cudaMallocHost(&e->pinned[p], total * 2));
    e->pinned_cap[p] = total * 2;
  }
  if (total > e->stage_cap[p]) {
    DLP_CUDA_TRY(cudaStreamSynchronize(e->stream));
    cudaFree(e->stage_dev[p]);
    e->stage_dev[p] = nullptr;
    e->stage_cap[p] = 0;
    DLP_CUDA_TRY(cudaMalloc(&e->stage_dev[p], total * 2));
    e->stage_cap[p] = total * 2;
  }
  char *hp = e->pinned[p], *dp = e->stage_dev[p];
  size_t off = 0;
  auto put = [&](const void *src, size_t bytes) {
    if (bytes) std::memcpy(hp + off, src, bytes);
    const void *r = dp + off;
    off += align16(bytes);
    return r;
  };
  dv.resize(count);
  for (int i = 0; i < count; ++i) {
    const dlp_batch_view &b = h[i];
    dlp_batch_view &o = dv[i];
    o.inserted = static_cast<const int *>(put(b.inserted, 4 * static_cast<size_t>(b.num_inserted)));
    o.num_inserted = b.num_inserted;
    o.gt_ids = static_cast<const int *>(put(b.gt_ids, 4 * static_cast<size_t>(b.num_gt)));
    o.gt_labels = static_cast<const float *>(put(b.gt_labels, 4 * static_cast<size_t>(b.num_gt)));
    o.num_gt = b.num_gt;
    o.deleted = static_cast<const int *>(put(b.deleted, 4 * static_cast<size_t>(b.num_deleted)));
    o.num_deleted = b.num_deleted;
    o.edge_src = static_cast<const int *>(put(b.edge_src, 4 * static_cast<size_t>(b.num_edges)));
    o.edge_dst = static_cast<const int *>(put(b.edge_dst, 4 * static_cast<size_t>(b.num_edges)));
    o.edge_weight = static_cast<const float *>(put(b.edge_weight, 4 * static_cast<size_t>(b.num_edges)));
    o.num_edges = b.num_edges;
  }
  if (off) DLP_CUDA_TRY(cudaMemcpyAsync(dp, hp, off, cudaMemcpyHostToDevice, e->stream));
  DLP_CUDA_TRY(cudaEventRecord(e->pinned_free[p], e->stream));
  return DLP_OK;
}

// Allocates every device array of a graph of n vertices and m directed edges
// (always in the same order: snapshots rely on it) for graph id gid.
int alloc_graph(dlp_engine *e, int n, int64_t m, bool with_truth, bool with_bmap, int gid, GraphSlot **out) {
  GraphSlot *g = new GraphSlot();
  g->n = n;
  g->m = m;
  g->has_truth = with_truth;
  g->has_bmap = with_bmap;
  DevState &d = g->st;
  d.n = n;
  int *full_row = nullptr;
  int2 *full_adj = nullptr;
  uint8_t *truth = nullptr;
  int *bmap = nullptr;
  auto &o = g->owned;
  size_t &b = g->bytes;
  std::vector<size_t> *z = &g->sizes;
  int st = DLP_OK;
  if ((st = dalloc(&full_row, n + 1, o, b, z)) || (st = dalloc(&full_adj, m, o, b, z)) ||
      (st = dalloc(&d.act_adj, m, o, b, z)) || (st = dalloc(&d.act_len, n, o, b, z)) ||
      (st = dalloc(&d.status, n, o, b, z)) || (st = dalloc(&d.gt, n, o, b, z)) ||
      (st = dalloc(&d.contrib, n, o, b, z)) || (st = dalloc(&d.lab0, n, o, b, z)) ||
      (st = dalloc(&d.lab1, n, o, b, z)) || (st = dalloc(&d.local, n, o, b, z)) ||
      (st = dalloc(&d.del_stamp, n, o, b, z)) || (st = dalloc(&d.gt_stamp, n, o, b, z)) ||
      (st = dalloc(&d.dirty_stamp, n, o, b, z)) || (st = dalloc(&d.front_stamp, n, o, b, z)) ||
      (st = dalloc(&d.dirty_list, n, o, b, z)) || (st = dalloc(&d.seed_list, n, o, b, z)) ||
      (st = dalloc(&d.flist, 3 * static_cast<size_t>(n), o, b, z)) ||
      (st = dalloc(&d.touched, 2 * static_cast<size_t>(n), o, b, z)) || (st = dalloc(&d.par, n, o, b, z)) ||
      (st = dalloc(&d.acc, 2 * static_cast<size_t>(n), o, b, z)) || (st = dalloc(&g->stats, kStepRing, o, b, z)) ||
      (st = dalloc(&d.nmeta, n, o, b, z)) || (st = dalloc(&d.rowinfo, n, o, b, z)) ||
      (with_truth && (st = dalloc(&truth, n, o, b, z))) || (with_bmap && (st = dalloc(&bmap, n, o, b, z))) ||
      (e->cfg.record &&
       ((st = dalloc(&d.rec_front0, n, o, b, z)) || (st = dalloc(&d.rec_root, n, o, b, z)) ||
        (st = dalloc(&d.rec_init, n, o, b, z)) || (st = dalloc(&d.rec_fsizes, dlp::session::kRecordIters, o, b, z)) ||
        (st = dalloc(&d.rec_minid, n, o, b, z))))) {
    g->free_all();
    delete g;
    return st;
  }
  d.full_row = full_row;
  d.full_adj = full_adj;
  d.truth = truth;
  d.batch_map = bmap;
  d.ctl = e->ctl_all + gid;
  *out = g;
  return DLP_OK;
}

int find_seq(GraphSlot *g, int batch) {
  for (int q = static_cast<int>(g->seq_batch.size()) - 1; q >= 0; --q)
    if (g->seq_batch[q] == batch) return q;
  return -1;
}

}  // namespace

extern "C" {

void dlp_config_default(dlp_config *cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->tau = -1.0f;
  cfg->delta = 1e-4f;
  cfg->max_iterations = 100000;
  cfg->semantics = DLP_SEMANTICS_REF;
  cfg->wait_timeout_s = 2.0;
  cfg->small_frontier_solo = 7;
}

int dlp_engine_create(const dlp_config *cfg_in, int max_graphs, size_t memory_budget_bytes, dlp_engine **out) {
  dlp::clear_error();
  if (!out) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null out");
  *out = nullptr;
  dlp_config cfg;
  if (cfg_in) cfg = *cfg_in;
  else dlp_config_default(&cfg);
  if (max_graphs <= 0 || max_graphs > dlp::engine::kMaxGraphs)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "max_graphs must be in [1, 1024]");
  if (!(cfg.delta > 0.0f)) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "delta must be positive");
  const int lanes = cfg.narrow_lanes == 0 ? 8 : cfg.narrow_lanes;
  if (lanes != 1 && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "narrow_lanes must be 1, 4, 8, 16 or 32");
  if (cfg.arithmetic != DLP_ARITH_IEEE && cfg.arithmetic != DLP_ARITH_REFERENCE_FAST_MATH)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "arithmetic must be DLP_ARITH_IEEE or DLP_ARITH_REFERENCE_FAST_MATH");
  if (cfg.solo_entry < 0 || cfg.solo_entry > dlp::engine::kSoloEntryMax || cfg.subgrid_entry < 0 ||
      cfg.subgrid_entry > dlp::engine::kSubEntryMax)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "solo_entry must be in [0, 1024] and subgrid_entry in [0, 4096]");
  DLP_CUDA_TRY(cudaSetDevice(cfg.device));
  DLP_TRY(dlp::require_device());
  dlp_engine *e = new dlp_engine();
  e->cfg = cfg;
  e->device = cfg.device;
  e->max_graphs = max_graphs;
  e->budget = memory_budget_bytes;
  e->lanes = lanes;
  e->kernel = dlp::engine::engine_kernel_ptr(lanes);
  auto bail = [&](int st) {
    delete e;
    return st;
  };
  if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(dlp::fail(DLP_ERR_CUDA, "stream creation failed"));
  for (int i = 0; i < kStepRing; ++i) {
    cudaEventCreate(&e->ev[i][0]);
    cudaEventCreate(&e->ev[i][1]);
  }
  e->ev_made = true;
  for (int i = 0; i < 2; ++i) {
    cudaEventCreateWithFlags(&e->recs_free[i], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&e->pinned_free[i], cudaEventDisableTiming);
    if (cudaMallocHost(&e->recs_host[i], sizeof(GraphRec) * max_graphs) != cudaSuccess)
      return bail(dlp::fail(DLP_ERR_OUT_OF_MEMORY, "pinned host allocation failed"));
  }
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg.device);
  e->smem = dlp::engine::engine_dynamic_smem();
  if (cudaFuncSetAttribute(e->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(e->smem)) !=
      cudaSuccess)
    return bail(dlp::fail(DLP_ERR_CUDA, "could not reserve the engine kernel's shared memory"));
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, e->kernel, dlp::session::kBlock, e->smem) !=
          cudaSuccess ||
      per_sm <= 0)
    return bail(dlp::fail(DLP_ERR_CUDA, "occupancy query failed for the engine kernel"));
  if (cfg.blocks_per_sm > 0) per_sm = std::min(per_sm, cfg.blocks_per_sm);
  e->grid = sms * per_sm;
  int st = DLP_OK;
  if ((st = dalloc(&e->ectl, 1, e->owned, e->owned_bytes)) ||
      (st = dalloc(&e->ctl_all, max_graphs, e->owned, e->owned_bytes)) ||
      (st = dalloc(&e->bc_all, max_graphs, e->owned, e->owned_bytes)) ||
      (st = dalloc(&e->recs_dev, 2 * static_cast<size_t>(max_graphs), e->owned, e->owned_bytes)) ||
      (st = dalloc(&e->progress_dev, max_graphs, e->owned, e->owned_bytes)))
    return bail(st);
  if (cudaMallocHost(&e->progress_host, sizeof(int2) * max_graphs) != cudaSuccess)
    return bail(dlp::fail(DLP_ERR_OUT_OF_MEMORY, "pinned host allocation failed"));
  if (cudaMemset(e->ectl, 0, sizeof(EngineCtl)) != cudaSuccess ||
      cudaMemset(e->ctl_all, 0, sizeof(SessionCtl) * max_graphs) != cudaSuccess ||
      cudaMemset(e->bc_all, 0, sizeof(BatchCounters) * max_graphs) != cudaSuccess)
    return bail(dlp::fail(DLP_ERR_CUDA, "initialisation failed"));
  e->graphs.assign(max_graphs, nullptr);
  e->held.assign(max_graphs, 0);
  *out = e;
  return DLP_OK;
}

int dlp_engine_destroy(dlp_engine *e) {
  delete e;
  return DLP_OK;
}

size_t dlp_engine_graph_bytes(int num_nodes, int64_t num_edges, int with_truth, int with_batch_map, int record) {
  return graph_bytes(num_nodes, num_edges, with_truth != 0, with_batch_map != 0, record != 0);
}

size_t dlp_engine_bytes_in_use(const dlp_engine *e) { return e ? e->used : 0; }

int dlp_engine_add_graph(dlp_engine *e, int n, int64_t m, const int *row_ptr, const int *col_ind,
                         const float *values, const float *true_labels, const int *vertex_batch_map,
                         int *graph_id) {
  dlp::clear_error();
  if (!e || !graph_id) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  *graph_id = -1;
  if (n <= 0 || m < 0 || m > 0x7fffffffLL || !row_ptr || (m > 0 && (!col_ind || !values)))
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "invalid graph arrays");
  if (row_ptr[0] != 0 || row_ptr[n] != m)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "row_ptr must start at 0 and end at num_edges");
  for (int i = 0; i < n; ++i)
    if (row_ptr[i + 1] < row_ptr[i]) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "row_ptr not monotone");
  for (int64_t k = 0; k < m; ++k)
    if (col_ind[k] >= n) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "col_ind out of range");
  const size_t need = graph_bytes(n, m, true_labels != nullptr, vertex_batch_map != nullptr, e->cfg.record != 0);
  if (e->budget > 0 && e->used + need > e->budget)
    return dlp::fail(DLP_ERR_OUT_OF_MEMORY, "graph does not fit the engine's device-memory budget (" +
                                                std::to_string(e->used + need) + " > " + std::to_string(e->budget) +
                                                " bytes)");
  int gid = -1;
  for (int i = 0; i < e->max_graphs; ++i)
    if (!e->graphs[i] && !e->held[i]) {
      gid = i;
      break;
    }
  if (gid < 0) return dlp::fail(DLP_ERR_OUT_OF_MEMORY, "the engine holds max_graphs graphs already");
  DLP_CUDA_TRY(cudaSetDevice(e->device));
  GraphSlot *g = nullptr;
  DLP_TRY(alloc_graph(e, n, m, true_labels != nullptr, vertex_batch_map != nullptr, gid, &g));
  g->tau = e->cfg.tau < 0.0f ? dlp_mean_edge_weight(m, col_ind, values) : e->cfg.tau;
  auto bail = [&](int st) {
    g->free_all();
    delete g;
    return st;
  };
  DevState &d = g->st;
  int *full_row = const_cast<int *>(d.full_row);
  int2 *full_adj = const_cast<int2 *>(d.full_adj);
  uint8_t *truth = const_cast<uint8_t *>(d.truth);
  int *bmap = const_cast<int *>(d.batch_map);
  int st = DLP_OK;
  auto up = [&](void *dst, const void *src, size_t bytes) -> int {
    if (bytes == 0) return DLP_OK;
    DLP_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return DLP_OK;
  };
  if ((st = up(full_row, row_ptr, sizeof(int) * (n + 1)))) return bail(st);
  if (m > 0) {
    int *col_tmp = nullptr;
    float *val_tmp = nullptr;
    if (cudaMalloc(&col_tmp, sizeof(int) * m) != cudaSuccess || cudaMalloc(&val_tmp, sizeof(float) * m) != cudaSuccess) {
      cudaFree(col_tmp);
      cudaFree(val_tmp);
      cudaGetLastError();
      return bail(dlp::fail(DLP_ERR_OUT_OF_MEMORY, "staging of the full graph failed"));
    }
    st = up(col_tmp, col_ind, sizeof(int) * m);
    if (!st) st = up(val_tmp, values, sizeof(float) * m);
    if (!st) {
      interleave_kernel<<<1024, 256, 0, e->stream>>>(col_tmp, val_tmp, full_adj, m);
      if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(e->stream) != cudaSuccess)
        st = dlp::fail(DLP_ERR_CUDA, "interleave of the full graph failed");
    }
    cudaFree(col_tmp);
    cudaFree(val_tmp);
    if (st) return bail(st);
  }
  if (truth) {
    std::vector<uint8_t> t(n);
    for (int i = 0; i < n; ++i) t[i] = true_labels[i] >= 0.5f ? 1 : 0;
    if ((st = up(truth, t.data(), n))) return bail(st);
  }
  if (bmap && (st = up(bmap, vertex_batch_map, sizeof(int) * n))) return bail(st);
  if ((st = reset_graph(e, g, gid))) return bail(st);
  e->graphs[gid] = g;
  e->used += g->bytes;
  *graph_id = gid;
  return DLP_OK;
}

int dlp_engine_remove_graph(dlp_engine *e, int graph_id) {
  dlp::clear_error();
  GraphSlot *g = slot_of(e, graph_id);
  if (!g) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "unknown graph id");
  DLP_CUDA_TRY(cudaSetDevice(e->device));
  DLP_CUDA_TRY(cudaStreamSynchronize(e->stream));
  if (g->inflight) --e->inflight;
  e->used -= std::min(e->used, g->bytes);
  g->free_all();
  delete g;
  e->graphs[graph_id] = nullptr;
  return DLP_OK;
}

// Snapshot layout: SnapHeader, the byte size of each device array (uint64),
// SessionCtl, BatchCounters, the arrays in allocation order, the previous
// batch's deletions (int32[prev_d]) and the batch index of every applied
// batch (int32[seq]).
namespace {
constexpr uint64_t kSnapMagic = 0x31504e5350444c44ull;  // "DLDPSNP1"
struct SnapHeader {
  uint64_t magic;
  int64_t m;
  int n, truth, bmap, record, semantics, narrays, seq, prev_d, last_inserted;
  float tau;
};

size_t snapshot_bytes(const GraphSlot *g) {
  size_t b = sizeof(SnapHeader) + sizeof(uint64_t) * g->sizes.size() + sizeof(SessionCtl) + sizeof(BatchCounters);
  for (size_t z : g->sizes) b += z;
  return b + sizeof(int) * (static_cast<size_t>(g->prev_d) + g->seq);
}
}  // namespace

int dlp_engine_snapshot(dlp_engine *e, int graph_id, void *out, size_t capacity, size_t *bytes) {
  dlp::clear_error();
  GraphSlot *g = slot_of(e, graph_id);
  if (!g || !bytes) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "unknown graph or null bytes");
  if (g->inflight) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "the graph's batch is still in progress");
  const size_t need = snapshot_bytes(g);
  *bytes = need;
  if (!out) return DLP_OK;
  if (capacity < need) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "snapshot buffer too small");
  DLP_CUDA_TRY(cudaSetDevice(e->device));
  DLP_CUDA_TRY(cudaStreamSynchronize(e->stream));
  char *p = static_cast<char *>(out);
  SnapHeader h{};
  h.magic = kSnapMagic;
  h.m = g->m;
  h.n = g->n;
  h.truth = g->has_truth;
  h.bmap = g->has_bmap;
  h.record = e->cfg.record != 0;
  h.semantics = e->cfg.semantics;
  h.narrays = static_cast<int>(g->sizes.size());
  h.seq = g->seq;
  h.prev_d = g->prev_d;
  h.last_inserted = g->last_inserted;
  h.tau = g->tau;
  std::memcpy(p, &h, sizeof(h));
  p += sizeof(h);
  for (size_t z : g->sizes) {
    const uint64_t v = z;
    std::memcpy(p, &v, sizeof(v));
    p += sizeof(v);
  }
  DLP_CUDA_TRY(cudaMemcpy(p, e->ctl_all + graph_id, sizeof(SessionCtl), cudaMemcpyDeviceToHost));
  p += sizeof(SessionCtl);
  DLP_CUDA_TRY(cudaMemcpy(p, e->bc_all + graph_id, sizeof(BatchCounters), cudaMemcpyDeviceToHost));
  p += sizeof(BatchCounters);
  for (size_t i = 0; i < g->owned.size(); ++i) {
    DLP_CUDA_TRY(cudaMemcpy(p, g->owned[i], g->sizes[i], cudaMemcpyDeviceToHost));
    p += g->sizes[i];
  }
  if (g->prev_d > 0) DLP_CUDA_TRY(cudaMemcpy(p, g->del_keep, sizeof(int) * g->prev_d, cudaMemcpyDeviceToHost));
  p += sizeof(int) * g->prev_d;
  if (g->seq > 0) std::memcpy(p, g->seq_batch.data(), sizeof(int) * g->seq);
  return DLP_OK;
}

namespace {
// Restores into graph id `want` (a free id), or into the first free id when
// want < 0.
int restore_graph(dlp_engine *e, const void *snapshot, size_t bytes, int want, int *graph_id) {
  *graph_id = -1;
  SnapHeader h{};
  if (bytes < sizeof(h)) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "snapshot too short");
  std::memcpy(&h, snapshot, sizeof(h));
  if (h.magic != kSnapMagic) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "not a graph snapshot");
  if (h.record != (e->cfg.record != 0) || h.semantics != e->cfg.semantics)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "snapshot was taken by an engine with other settings");
  if (h.n <= 0 || h.m < 0 || h.seq < 0 || h.prev_d < 0 || h.narrays <= 0)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "corrupt snapshot header");
  const size_t need = graph_bytes(h.n, h.m, h.truth != 0, h.bmap != 0, h.record != 0);
  if (e->budget > 0 && e->used + need > e->budget)
    return dlp::fail(DLP_ERR_OUT_OF_MEMORY, "graph does not fit the engine's device-memory budget");
  int gid = -1;
  if (want >= 0) {
    if (want >= e->max_graphs || e->graphs[want])
      return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "graph id " + std::to_string(want) + " is not free");
    gid = want;
  } else {
    for (int i = 0; i < e->max_graphs; ++i)
      if (!e->graphs[i] && !e->held[i]) {
        gid = i;
        break;
      }
  }
  if (gid < 0) return dlp::fail(DLP_ERR_OUT_OF_MEMORY, "the engine holds max_graphs graphs already");
  DLP_CUDA_TRY(cudaSetDevice(e->device));
  GraphSlot *g = nullptr;
  DLP_TRY(alloc_graph(e, h.n, h.m, h.truth != 0, h.bmap != 0, gid, &g));
  auto bail = [&](int st) {
    g->free_all();
    delete g;
    return st;
  };
  if (static_cast<int>(g->sizes.size()) != h.narrays)
    return bail(dlp::fail(DLP_ERR_INVALID_ARGUMENT, "snapshot layout does not match this build"));
  const char *p = static_cast<const char *>(snapshot) + sizeof(h);
  for (size_t z : g->sizes) {
    uint64_t v = 0;
    std::memcpy(&v, p, sizeof(v));
    p += sizeof(v);
    if (v != z) return bail(dlp::fail(DLP_ERR_INVALID_ARGUMENT, "snapshot layout does not match this build"));
  }
  g->tau = h.tau;
  g->seq = h.seq;
  g->last_inserted = h.last_inserted;
  g->prev_d = h.prev_d;  // del_keep is still null, so growing it below copies nothing
  if (bytes < snapshot_bytes(g)) return bail(dlp::fail(DLP_ERR_INVALID_ARGUMENT, "snapshot too short"));
  int st = DLP_OK;
  auto up = [&](void *dst, const void *src, size_t n) -> int {
    DLP_CUDA_TRY(cudaMemcpy(dst, src, n, cudaMemcpyHostToDevice));
    return DLP_OK;
  };
  if ((st = up(e->ctl_all + gid, p, sizeof(SessionCtl)))) return bail(st);
  p += sizeof(SessionCtl);
  if ((st = up(e->bc_all + gid, p, sizeof(BatchCounters)))) return bail(st);
  p += sizeof(BatchCounters);
  for (size_t i = 0; i < g->owned.size(); ++i) {
    if ((st = up(g->owned[i], p, g->sizes[i]))) return bail(st);
    p += g->sizes[i];
  }
  if ((st = grow_graph_scratch(e, g, 0, h.prev_d))) return bail(st);
  if (h.prev_d > 0 && (st = up(g->del_keep, p, sizeof(int) * h.prev_d))) return bail(st);
  p += sizeof(int) * h.prev_d;
  g->seq_batch.assign(reinterpret_cast<const int *>(p), reinterpret_cast<const int *>(p) + h.seq);
  g->seq_step.assign(h.seq, -1);
  e->graphs[gid] = g;
  e->held[gid] = 0;
  e->used += g->bytes;
  *graph_id = gid;
  return DLP_OK;
}
}  // namespace

int dlp_engine_restore(dlp_engine *e, const void *snapshot, size_t bytes, int *graph_id) {
  dlp::clear_error();
  if (!e || !snapshot || !graph_id) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  return restore_graph(e, snapshot, bytes, -1, graph_id);
}

int dlp_engine_restore_as(dlp_engine *e, const void *snapshot, size_t bytes, int graph_id) {
  dlp::clear_error();
  if (!e || !snapshot || graph_id < 0) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument or negative id");
  int got = -1;
  return restore_graph(e, snapshot, bytes, graph_id, &got);
}

int dlp_engine_hold_id(dlp_engine *e, int graph_id) {
  dlp::clear_error();
  if (!e || graph_id < 0 || graph_id >= e->max_graphs) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "bad graph id");
  if (e->graphs[graph_id]) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "graph id is in use");
  e->held[graph_id] = 1;
  return DLP_OK;
}

int dlp_engine_release_id(dlp_engine *e, int graph_id) {
  dlp::clear_error();
  if (!e || graph_id < 0 || graph_id >= e->max_graphs) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "bad graph id");
  e->held[graph_id] = 0;
  return DLP_OK;
}

size_t dlp_engine_graph_resident_bytes(const dlp_engine *e, int graph_id) {
  GraphSlot *g = slot_of(const_cast<dlp_engine *>(e), graph_id);
  return g ? g->bytes : 0;
}

int dlp_engine_reset_graph(dlp_engine *e, int graph_id) {
  dlp::clear_error();
  GraphSlot *g = slot_of(e, graph_id);
  if (!g) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "unknown graph id");
  DLP_CUDA_TRY(cudaSetDevice(e->device));
  DLP_TRY(reset_graph(e, g, graph_id));
  int zero = 0;
  DLP_CUDA_TRY(cudaMemcpy(&e->ectl->err, &zero, sizeof(int), cudaMemcpyHostToDevice));
  return DLP_OK;
}

float dlp_engine_tau(const dlp_engine *e, int graph_id) {
  GraphSlot *g = slot_of(const_cast<dlp_engine *>(e), graph_id);
  return g ? g->tau : 0.0f;
}

void *dlp_engine_stream(dlp_engine *e) { return e ? static_cast<void *>(e->stream) : nullptr; }

int dlp_engine_step(dlp_engine *e, int count, const int *graph_ids, const int *batch_indices,
                    const dlp_batch_view *host_batches, dlp_batch_stats *stats) {
  dlp::clear_error();
  if (!e || count < 0 || (count > 0 && (!graph_ids || !batch_indices || !host_batches)))
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  DLP_CUDA_TRY(cudaSetDevice(e->device));
  std::vector<dlp_batch_view> dv;
  DLP_TRY(stage_step(e, count, graph_ids, host_batches, dv));
  DLP_TRY(launch_step(e, count, graph_ids, batch_indices, dv.data()));
  if (stats) {
    DLP_TRY(dlp_engine_synchronize(e));
    for (int i = 0; i < count; ++i) DLP_TRY(dlp_engine_stats(e, graph_ids[i], batch_indices[i], stats + i));
  }
  return DLP_OK;
}

int dlp_engine_step_device(dlp_engine *e, int count, const int *graph_ids, const int *batch_indices,
                           const dlp_batch_view *device_batches) {
  dlp::clear_error();
  if (!e || count < 0 || (count > 0 && (!graph_ids || !batch_indices || !device_batches)))
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  DLP_CUDA_TRY(cudaSetDevice(e->device));
  return launch_step(e, count, graph_ids, batch_indices, device_batches);
}

int dlp_engine_step_sliced(dlp_engine *e, int count, const int *graph_ids, const int *batch_indices,
                           const dlp_batch_view *device_batches, int pass_budget, double slice_us,
                           int *finished_ids, int *num_finished, int *num_continuing) {
  dlp::clear_error();
  if (!e || count < 0 || (count > 0 && (!graph_ids || !batch_indices || !device_batches)) || !num_finished)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  if (pass_budget < 0 || !(slice_us >= 0.0)) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "negative budget");
  *num_finished = 0;
  if (num_continuing) *num_continuing = e->inflight;
  DLP_CUDA_TRY(cudaSetDevice(e->device));
  SliceOpts o;
  o.pass_budget = pass_budget;
  o.slice_ns = static_cast<unsigned long long>(slice_us * 1e3);
  o.resume = true;
  e->last_finished.clear();
  DLP_TRY(launch_step(e, count, graph_ids, batch_indices, device_batches, o));
  *num_finished = static_cast<int>(e->last_finished.size());
  if (finished_ids) std::copy(e->last_finished.begin(), e->last_finished.end(), finished_ids);
  if (num_continuing) *num_continuing = e->inflight;
  return DLP_OK;
}

int dlp_engine_reserve(dlp_engine *e, int graph_id, int max_edges, int max_deleted) {
  dlp::clear_error();
  GraphSlot *g = slot_of(e, graph_id);
  if (!g || max_edges < 0 || max_deleted < 0) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "unknown graph or negative size");
  DLP_CUDA_TRY(cudaSetDevice(e->device));
  return grow_graph_scratch(e, g, max_edges, max_deleted);
}

int dlp_engine_graph_nodes(const dlp_engine *e, int graph_id) {
  GraphSlot *g = slot_of(const_cast<dlp_engine *>(e), graph_id);
  return g ? g->n : -1;
}

int dlp_engine_in_progress(const dlp_engine *e, int graph_id) {
  GraphSlot *g = slot_of(const_cast<dlp_engine *>(e), graph_id);
  return g && g->inflight ? 1 : 0;
}

int dlp_engine_synchronize(dlp_engine *e) {
  dlp::clear_error();
  if (!e) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null engine");
  DLP_CUDA_TRY(cudaSetDevice(e->device));
  DLP_CUDA_TRY(cudaStreamSynchronize(e->stream));
  return device_error(e);
}

int dlp_engine_stats(dlp_engine *e, int graph_id, int batch_index, dlp_batch_stats *out) {
  dlp::clear_error();
  GraphSlot *g = slot_of(e, graph_id);
  if (!g || !out) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "unknown graph or null out");
  const int seq = find_seq(g, batch_index);
  if (seq < 0 || g->seq - seq > kStepRing) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "no statistics kept for that batch");
  if (g->inflight && seq == g->seq - 1) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "that batch is still in progress");
  DLP_CUDA_TRY(cudaSetDevice(e->device));
  DLP_CUDA_TRY(cudaStreamSynchronize(e->stream));
  DLP_TRY(device_error(e));
  DLP_CUDA_TRY(cudaMemcpy(out, g->stats + (seq % kStepRing), sizeof(*out), cudaMemcpyDeviceToHost));
  const int step = g->seq_step[seq];  // -1 for a batch applied before a restore
  float ms = 0.0f;
  if (step >= 0 && e->steps - step <= kStepRing &&
      cudaEventElapsedTime(&ms, e->ev[step % kStepRing][0], e->ev[step % kStepRing][1]) == cudaSuccess)
    out->device_ms = ms;
  else
    cudaGetLastError();
  return DLP_OK;
}

int dlp_engine_elapsed_ms(dlp_engine *e, int first_step, int last_step, float *ms) {
  dlp::clear_error();
  if (!e || !ms || first_step < 0 || last_step < first_step || last_step >= e->steps ||
      e->steps - first_step > kStepRing)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "no events kept for that step range");
  DLP_CUDA_TRY(cudaSetDevice(e->device));
  DLP_CUDA_TRY(cudaStreamSynchronize(e->stream));
  DLP_CUDA_TRY(cudaEventElapsedTime(ms, e->ev[first_step % kStepRing][0], e->ev[last_step % kStepRing][1]));
  return DLP_OK;
}

int dlp_engine_steps(const dlp_engine *e) { return e ? e->steps : 0; }

int dlp_engine_debug(dlp_engine *e, int *out4) {
  dlp::clear_error();
  if (!e || !out4) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  DLP_CUDA_TRY(cudaSetDevice(e->device));
  DLP_CUDA_TRY(cudaStreamSynchronize(e->stream));
  EngineCtl c;
  DLP_CUDA_TRY(cudaMemcpy(&c, e->ectl, sizeof(c), cudaMemcpyDeviceToHost));
  out4[0] = c.err;
  out4[1] = c.where;
  out4[2] = c.where_pass;
  out4[3] = std::max(c.solo_passes[0], c.solo_passes[1]);
  return DLP_OK;
}

int dlp_engine_pass_modes(dlp_engine *e, unsigned long long *passes4, double *seconds4) {
  dlp::clear_error();
  if (!e || !passes4 || !seconds4) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  DLP_CUDA_TRY(cudaSetDevice(e->device));
  DLP_CUDA_TRY(cudaStreamSynchronize(e->stream));
  EngineCtl c;
  DLP_CUDA_TRY(cudaMemcpy(&c, e->ectl, sizeof(c), cudaMemcpyDeviceToHost));
  for (int m = 0; m < 4; ++m) {
    passes4[m] = c.mode_passes[m];
    seconds4[m] = static_cast<double>(c.mode_ns[m]) * 1e-9;
  }
  return DLP_OK;
}

int dlp_engine_read_labels(dlp_engine *e, int graph_id, float *host_labels) {
  dlp::clear_error();
  GraphSlot *g = slot_of(e, graph_id);
  if (!g || !host_labels) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "unknown graph or null out");
  if (g->inflight) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "the graph's batch is still in progress");
  DLP_TRY(dlp_engine_synchronize(e));
  int cb = 0;
  DLP_CUDA_TRY(cudaMemcpy(&cb, &e->ctl_all[graph_id].cur_buf, sizeof(int), cudaMemcpyDeviceToHost));
  DLP_CUDA_TRY(cudaMemcpy(host_labels, cb ? g->st.lab1 : g->st.lab0, sizeof(float) * g->n, cudaMemcpyDeviceToHost));
  return DLP_OK;
}

int dlp_engine_artefact(dlp_engine *e, int graph_id, int which, void *host_out, int64_t capacity, int64_t *count) {
  dlp::clear_error();
  GraphSlot *g = slot_of(e, graph_id);
  if (!g || !count) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "unknown graph or null count");
  if (g->inflight) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "the graph's batch is still in progress");
  DLP_TRY(dlp_engine_synchronize(e));
  const DevState &d = g->st;
  BatchCounters bc{};
  if (g->seq > 0) DLP_CUDA_TRY(cudaMemcpy(&bc, e->bc_all + graph_id, sizeof(bc), cudaMemcpyDeviceToHost));
  dlp_batch_stats last{};
  if (g->seq > 0)
    DLP_CUDA_TRY(cudaMemcpy(&last, g->stats + (g->seq - 1) % kStepRing, sizeof(last), cudaMemcpyDeviceToHost));
  const bool rec = e->cfg.record != 0;
  const void *src = nullptr;
  int64_t cnt = 0;
  switch (which) {
    case DLP_ART_SEED_MARKS: src = d.seed_list; cnt = bc.num_seeds; break;
    case DLP_ART_FRONTIER0:
      if (!rec) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "engine was not created with record");
      src = d.rec_front0; cnt = bc.seed_frontier; break;
    case DLP_ART_SUB_EDGES: {
      const int64_t kept = bc.num_kept;
      *count = 4 * kept;
      if (host_out && kept > 0) {
        if (capacity < 4 * kept) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "capacity too small");
        std::vector<int> pr(2 * kept);
        DLP_CUDA_TRY(cudaMemcpy(pr.data(), g->sub_pairs, sizeof(int) * 2 * kept, cudaMemcpyDeviceToHost));
        int *o = static_cast<int *>(host_out);
        for (int64_t k = 0; k < kept; ++k) {
          o[4 * k] = pr[2 * k];
          o[4 * k + 1] = pr[2 * k + 1];
          o[4 * k + 2] = pr[2 * k + 1];
          o[4 * k + 3] = pr[2 * k];
        }
      }
      return DLP_OK;
    }
    case DLP_ART_COMP_ROOT:
    case DLP_ART_INIT_LABELS:
      if (!rec) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "engine was not created with record");
      src = which == DLP_ART_COMP_ROOT ? static_cast<const void *>(d.rec_root) : d.rec_init;
      cnt = g->last_inserted;
      break;
    case DLP_ART_FRONTIER_SIZES:
      if (!rec) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "engine was not created with record");
      src = d.rec_fsizes;
      cnt = std::min(last.iterations, dlp::session::kRecordIters);
      break;
    case DLP_ART_ROW_LENGTHS: src = d.act_len; cnt = g->n; break;
    case DLP_ART_LABELS: {
      *count = g->n;
      if (host_out) {
        if (capacity < g->n) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "capacity too small");
        return dlp_engine_read_labels(e, graph_id, static_cast<float *>(host_out));
      }
      return DLP_OK;
    }
    default: return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "unknown artefact");
  }
  *count = cnt;
  if (host_out && cnt > 0) {
    if (capacity < cnt) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "capacity too small");
    DLP_CUDA_TRY(cudaMemcpy(host_out, src, 4 * cnt, cudaMemcpyDeviceToHost));
  }
  return DLP_OK;
}

// -------------------------------------------------- one-graph session --------

int dlp_session_create(const dlp_config *cfg, int n, int64_t m, const int *row_ptr, const int *col_ind,
                       const float *values, const float *true_labels, const int *vertex_batch_map,
                       dlp_session **out) {
  dlp::clear_error();
  if (!out) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null out");
  *out = nullptr;
  dlp_engine *e = nullptr;
  DLP_TRY(dlp_engine_create(cfg, 1, 0, &e));
  int gid = -1;
  const int st = dlp_engine_add_graph(e, n, m, row_ptr, col_ind, values, true_labels, vertex_batch_map, &gid);
  if (st != DLP_OK) {
    const std::string msg = dlp_last_error();
    delete e;
    return dlp::fail(st, msg);
  }
  dlp_session *s = new dlp_session();
  s->eng = e;
  s->gid = gid;
  *out = s;
  return DLP_OK;
}

int dlp_session_destroy(dlp_session *s) {
  if (s) {
    delete s->eng;
    delete s;
  }
  return DLP_OK;
}

int dlp_session_reset(dlp_session *s) {
  if (!s) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null session");
  return dlp_engine_reset_graph(s->eng, s->gid);
}

float dlp_session_tau(const dlp_session *s) { return s ? dlp_engine_tau(s->eng, s->gid) : 0.0f; }
void *dlp_session_stream(dlp_session *s) { return s ? dlp_engine_stream(s->eng) : nullptr; }

int dlp_session_apply_batch(dlp_session *s, int batch_index, const dlp_batch_view *host_batch,
                            dlp_batch_stats *stats) {
  if (!s || !host_batch) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  return dlp_engine_step(s->eng, 1, &s->gid, &batch_index, host_batch, stats);
}

int dlp_session_apply_batch_device(dlp_session *s, int batch_index, const dlp_batch_view *device_batch) {
  if (!s || !device_batch) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  return dlp_engine_step_device(s->eng, 1, &s->gid, &batch_index, device_batch);
}

int dlp_session_synchronize(dlp_session *s) {
  if (!s) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null session");
  return dlp_engine_synchronize(s->eng);
}

int dlp_session_stats(dlp_session *s, int batch_index, dlp_batch_stats *out) {
  if (!s) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null session");
  return dlp_engine_stats(s->eng, s->gid, batch_index, out);
}

int dlp_session_elapsed_ms(dlp_session *s, int first, int last, float *ms) {
  dlp::clear_error();
  if (!s) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null session");
  GraphSlot *g = slot_of(s->eng, s->gid);
  const int a = find_seq(g, first), b = find_seq(g, last);
  if (a < 0 || b < 0 || b < a) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "no events kept for that batch range");
  return dlp_engine_elapsed_ms(s->eng, g->seq_step[a], g->seq_step[b], ms);
}

int dlp_session_read_labels(dlp_session *s, float *host_labels) {
  if (!s) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null session");
  return dlp_engine_read_labels(s->eng, s->gid, host_labels);
}

int dlp_session_pass_modes(dlp_session *s, unsigned long long *passes4, double *seconds4) {
  dlp::clear_error();
  if (!s) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null session");
  return dlp_engine_pass_modes(s->eng, passes4, seconds4);
}

int dlp_session_debug(dlp_session *s, int *out4) {
  if (!s) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null session");
  return dlp_engine_debug(s->eng, out4);
}

int dlp_session_artefact(dlp_session *s, int which, void *host_out, int64_t capacity, int64_t *count) {
  if (!s) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null session");
  return dlp_engine_artefact(s->eng, s->gid, which, host_out, capacity, count);
}

}  // extern "C"
