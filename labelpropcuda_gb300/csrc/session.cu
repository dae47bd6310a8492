// Host side of the resident session (C ABI group 2 in dlp_gb300.h).
//
// Memory layout in HBM, per session (n vertices, m directed full-graph edges):
//   full_row  int32[n+1]     full_adj int2[m] {col, weight bits}
//   act_adj   int2[m]        live rows in the same slots as full_adj
//   act_len   int32[n]       live row length
//   status/gt int8[n]        truth uint8[n]       contrib int32[n]
//   lab0/lab1 fp32[n]        the stale double buffer of the reference
//   stamps    uint32[n] x 4  (deleted, ground truth, dirty, frontier)
//   lists     int32: dirty[n], seeds[n], frontier 3 x [n], touched 2 x [n]
//   SV        par int32[n], acc int64[2n]
//   per batch edge scratch sized by the largest batch seen
// Nothing is O(n) per batch: every pass walks the batch's lists, the rows next
// to changed vertices, and the frontier.
#include <algorithm>
#include <cstring>
#include <vector>

#include "session_kernel.cuh"

namespace dlp {
namespace session {
const void *batch_kernel_ptr(int lanes);
}
}  // namespace dlp

using dlp::session::BatchArgs;
using dlp::session::BatchCounters;
using dlp::session::DevState;
using dlp::session::SessionCtl;

namespace {

constexpr int kStatsRing = 4096;

__global__ void interleave_kernel(const int *col, const float *val, int2 *adj, int64_t m) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < m;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    adj[i] = make_int2(col[i], __float_as_int(val[i]));
}

__global__ void fill_f32_kernel(float *p, float v, int64_t count) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    p[i] = v;
}

size_t align16(size_t x) { return (x + 15) & ~static_cast<size_t>(15); }

template <class T>
int dalloc(T **p, size_t count, std::vector<void *> &owned) {
  void *q = nullptr;
  const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return dlp::fail(e == cudaErrorMemoryAllocation ? DLP_ERR_OUT_OF_MEMORY : DLP_ERR_CUDA,
                     std::string("cudaMalloc of ") + std::to_string(bytes) + " bytes failed: " +
                         cudaGetErrorString(e));
  }
  owned.push_back(q);
  *p = static_cast<T *>(q);
  return DLP_OK;
}

}  // namespace

struct dlp_session {
  dlp_config cfg;
  int device = 0;
  int n = 0;
  int64_t m = 0;
  float tau = 0.5f;
  int lanes = 8;
  int grid = 0;
  const void *kernel = nullptr;
  cudaStream_t stream = nullptr;
  std::vector<void *> owned;  // fixed-size device allocations
  DevState st{};
  SessionCtl *ctl = nullptr;
  BatchCounters *bc = nullptr;
  dlp_batch_stats *stats = nullptr;  // device ring
  // per-batch edge scratch (grown)
  int edge_cap = 0;
  int *lsrc = nullptr, *ldst = nullptr, *sub_pairs = nullptr, *sub_local = nullptr;
  int del_cap = 0;
  int *del_pre = nullptr;
  // host-mode staging: two device sets (the previous batch's deletions stay
  // readable) and one pinned host buffer
  size_t stage_cap[2] = {0, 0};
  char *stage_dev[2] = {nullptr, nullptr};
  size_t pinned_cap = 0;
  char *pinned = nullptr;
  // batch bookkeeping
  int seq = 0;
  int last_inserted = 0;
  const int *prev_del = nullptr;
  int prev_del_n = 0;
  std::vector<int> seq_batch;  // caller's batch index per seq
  cudaEvent_t ev[kStatsRing][2];
  bool ev_made = false;

  ~dlp_session() {
    if (device >= 0) cudaSetDevice(device);
    for (void *p : owned) cudaFree(p);
    cudaFree(lsrc);
    cudaFree(ldst);
    cudaFree(sub_pairs);
    cudaFree(sub_local);
    cudaFree(del_pre);
    cudaFree(stage_dev[0]);
    cudaFree(stage_dev[1]);
    if (pinned) cudaFreeHost(pinned);
    if (ev_made)
      for (int i = 0; i < kStatsRing; ++i) {
        cudaEventDestroy(ev[i][0]);
        cudaEventDestroy(ev[i][1]);
      }
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

int grow_edges(dlp_session *s, int need) {
  if (need <= s->edge_cap) return DLP_OK;
  int cap = std::max(need, std::max(1024, s->edge_cap * 2));
  cap = (cap + 3) & ~3;
  DLP_CUDA_TRY(cudaStreamSynchronize(s->stream));
  cudaFree(s->lsrc);
  cudaFree(s->ldst);
  cudaFree(s->sub_pairs);
  cudaFree(s->sub_local);
  s->lsrc = s->ldst = s->sub_pairs = s->sub_local = nullptr;
  s->edge_cap = 0;
  DLP_CUDA_TRY(cudaMalloc(&s->lsrc, sizeof(int) * cap));
  DLP_CUDA_TRY(cudaMalloc(&s->ldst, sizeof(int) * cap));
  DLP_CUDA_TRY(cudaMalloc(&s->sub_pairs, sizeof(int) * 2 * static_cast<size_t>(cap)));
  DLP_CUDA_TRY(cudaMalloc(&s->sub_local, sizeof(int) * 2 * static_cast<size_t>(cap)));
  s->edge_cap = cap;
  return DLP_OK;
}

int grow_del(dlp_session *s, int need) {
  if (need <= s->del_cap) return DLP_OK;
  const int cap = std::max(need, std::max(1024, s->del_cap * 2));
  DLP_CUDA_TRY(cudaStreamSynchronize(s->stream));
  cudaFree(s->del_pre);
  s->del_pre = nullptr;
  s->del_cap = 0;
  DLP_CUDA_TRY(cudaMalloc(&s->del_pre, sizeof(int) * cap));
  s->del_cap = cap;
  return DLP_OK;
}

int check_ids(const int *ids, int count, int n, const char *what) {
  if (count < 0) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, std::string("negative count for ") + what);
  if (count > 0 && !ids) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, std::string("null ") + what);
  for (int i = 0; i < count; ++i)
    if (ids[i] < 0 || ids[i] >= n)
      return dlp::fail(DLP_ERR_INVALID_ARGUMENT, std::string("vertex id ") + std::to_string(ids[i]) +
                                                     " out of range in " + what);
  return DLP_OK;
}

int reset_state(dlp_session *s) {
  const int n = s->n;
  DevState &d = s->st;
  cudaStream_t q = s->stream;
  DLP_CUDA_TRY(cudaMemsetAsync(d.act_len, 0, sizeof(int) * n, q));
  DLP_CUDA_TRY(cudaMemsetAsync(d.status, dlp::kDeleted, n, q));
  DLP_CUDA_TRY(cudaMemsetAsync(d.gt, 0xff, n, q));
  DLP_CUDA_TRY(cudaMemsetAsync(d.contrib, 0xff, sizeof(int) * n, q));
  DLP_CUDA_TRY(cudaMemsetAsync(d.local, 0xff, sizeof(int) * n, q));
  for (unsigned *p : {d.del_stamp, d.gt_stamp, d.dirty_stamp, d.front_stamp})
    DLP_CUDA_TRY(cudaMemsetAsync(p, 0, sizeof(unsigned) * n, q));
  fill_f32_kernel<<<1024, 256, 0, q>>>(d.lab0, 0.5f, n);
  fill_f32_kernel<<<1024, 256, 0, q>>>(d.lab1, 0.5f, n);
  DLP_CUDA_TRY(cudaGetLastError());
  DLP_CUDA_TRY(cudaMemsetAsync(s->ctl, 0, sizeof(SessionCtl), q));
  DLP_CUDA_TRY(cudaStreamSynchronize(q));
  s->seq = 0;
  s->prev_del = nullptr;
  s->prev_del_n = 0;
  s->seq_batch.clear();
  return DLP_OK;
}

// Copies a host batch into one pinned buffer and one device staging set with
// a single H2D copy; returns device views.
int stage_batch(dlp_session *s, const dlp_batch_view *h, dlp_batch_view *dv) {
  const size_t sz_i = align16(sizeof(int) * h->num_inserted);
  const size_t sz_g = align16(sizeof(int) * h->num_gt);
  const size_t sz_gl = align16(sizeof(float) * h->num_gt);
  const size_t sz_d = align16(sizeof(int) * h->num_deleted);
  const size_t sz_e = align16(sizeof(int) * h->num_edges);
  const size_t total = sz_i + sz_g + sz_gl + sz_d + 3 * sz_e + 16;
  const int set = s->seq & 1;
  if (total > s->pinned_cap) {
    DLP_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (s->pinned) cudaFreeHost(s->pinned);
    s->pinned = nullptr;
    s->pinned_cap = 0;
    const size_t cap = std::max(total, s->pinned_cap * 2);
    DLP_CUDA_TRY(cudaMallocHost(&s->pinned, cap));
    s->pinned_cap = cap;
  }
  if (total > s->stage_cap[set]) {
    DLP_CUDA_TRY(cudaStreamSynchronize(s->stream));
    cudaFree(s->stage_dev[set]);
    s->stage_dev[set] = nullptr;
    s->stage_cap[set] = 0;
    const size_t cap = std::max(total, s->stage_cap[set] * 2);
    DLP_CUDA_TRY(cudaMalloc(&s->stage_dev[set], cap));
    s->stage_cap[set] = cap;
  }
  // The pinned buffer is reused: wait until the previous copy out of it is done.
  DLP_CUDA_TRY(cudaStreamSynchronize(s->stream));
  char *hp = s->pinned;
  char *dp = s->stage_dev[set];
  size_t off = 0;
  auto put = [&](const void *src, size_t bytes, size_t padded) {
    if (bytes) std::memcpy(hp + off, src, bytes);
    const void *r = dp + off;
    off += padded;
    return r;
  };
  dv->inserted = static_cast<const int *>(put(h->inserted, sizeof(int) * h->num_inserted, sz_i));
  dv->num_inserted = h->num_inserted;
  dv->gt_ids = static_cast<const int *>(put(h->gt_ids, sizeof(int) * h->num_gt, sz_g));
  dv->gt_labels = static_cast<const float *>(put(h->gt_labels, sizeof(float) * h->num_gt, sz_gl));
  dv->num_gt = h->num_gt;
  dv->deleted = static_cast<const int *>(put(h->deleted, sizeof(int) * h->num_deleted, sz_d));
  dv->num_deleted = h->num_deleted;
  dv->edge_src = static_cast<const int *>(put(h->edge_src, sizeof(int) * h->num_edges, sz_e));
  dv->edge_dst = static_cast<const int *>(put(h->edge_dst, sizeof(int) * h->num_edges, sz_e));
  dv->edge_weight = static_cast<const float *>(put(h->edge_weight, sizeof(float) * h->num_edges, sz_e));
  dv->num_edges = h->num_edges;
  if (off) DLP_CUDA_TRY(cudaMemcpyAsync(dp, hp, off, cudaMemcpyHostToDevice, s->stream));
  return DLP_OK;
}

int launch_batch(dlp_session *s, int batch_index, const dlp_batch_view *dv) {
  if (dv->num_inserted < 0 || dv->num_gt < 0 || dv->num_deleted < 0 || dv->num_edges < 0)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "negative batch size");
  // per-position arrays (SV parents, supernode sums) hold n entries
  if (dv->num_inserted > s->n)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "more inserted entries than vertices");
  if ((dv->num_inserted && !dv->inserted) || (dv->num_gt && (!dv->gt_ids || !dv->gt_labels)) ||
      (dv->num_deleted && !dv->deleted) ||
      (dv->num_edges && (!dv->edge_src || !dv->edge_dst || !dv->edge_weight)))
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null batch array");
  DLP_TRY(grow_edges(s, dv->num_edges));
  DLP_TRY(grow_del(s, dv->num_deleted));
  DevState d = s->st;
  d.lsrc = s->lsrc;
  d.ldst = s->ldst;
  d.sub_pairs = s->sub_pairs;
  d.sub_local = s->sub_local;
  d.del_pre = s->del_pre;
  const int slot = s->seq % kStatsRing;
  d.stats_slot = s->stats + slot;

  BatchArgs a{};
  a.batch = batch_index;
  a.seq = s->seq;
  a.ins = dv->inserted;
  a.I = dv->num_inserted;
  a.gt_ids = dv->gt_ids;
  a.gt_lab = dv->gt_labels;
  a.G = dv->num_gt;
  a.del = dv->deleted;
  a.D = dv->num_deleted;
  a.es = dv->edge_src;
  a.ed = dv->edge_dst;
  a.ew = dv->edge_weight;
  a.E = dv->num_edges;
  a.prev_del = s->prev_del;
  a.PD = s->prev_del_n;
  a.tau = s->tau;
  a.delta = s->cfg.delta;
  a.max_iter = s->cfg.max_iterations;
  a.spec = s->cfg.semantics == DLP_SEMANTICS_SPEC;
  a.record = s->cfg.record != 0;
  a.solo = s->cfg.small_frontier_solo != 0;
  const double to = s->cfg.wait_timeout_s > 0 ? s->cfg.wait_timeout_s : 2.0;
  a.timeout_ns = static_cast<unsigned long long>(to * 1e9);

  DLP_CUDA_TRY(cudaMemsetAsync(s->bc, 0, sizeof(BatchCounters), s->stream));
  DLP_CUDA_TRY(cudaEventRecord(s->ev[slot][0], s->stream));
  void *args[] = {&d, &a};
  DLP_TRY(dlp::launch_cooperative(s->kernel, s->grid, dlp::session::kBlock, args, 0, s->stream));
  DLP_CUDA_TRY(cudaEventRecord(s->ev[slot][1], s->stream));
  if (static_cast<int>(s->seq_batch.size()) <= s->seq) s->seq_batch.resize(s->seq + 1);
  s->seq_batch[s->seq] = batch_index;
  s->prev_del = dv->deleted;
  s->prev_del_n = dv->num_deleted;
  s->last_inserted = dv->num_inserted;
  ++s->seq;
  return DLP_OK;
}

int device_error(dlp_session *s) {
  int err = 0;
  DLP_CUDA_TRY(cudaMemcpy(&err, &s->ctl->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err != 0)
    return dlp::fail(err, std::string("device reported ") + dlp_status_string(err) +
                              "; the session must be reset");
  return DLP_OK;
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
  cfg->device = 0;
  cfg->record = 0;
  cfg->narrow_lanes = 0;
  cfg->blocks_per_sm = 0;
  cfg->wait_timeout_s = 2.0;
  cfg->small_frontier_solo = 1;
}

int dlp_session_create(const dlp_config *cfg_in, int n, int64_t m, const int *row_ptr,
                       const int *col_ind, const float *values, const float *true_labels,
                       const int *vertex_batch_map, dlp_session **out) {
  dlp::clear_error();
  if (!out) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null out");
  *out = nullptr;
  dlp_config cfg;
  if (cfg_in) cfg = *cfg_in;
  else dlp_config_default(&cfg);
  if (n <= 0 || m < 0 || m > 0x7fffffffLL || !row_ptr || (m > 0 && (!col_ind || !values)))
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "invalid graph arrays");
  if (row_ptr[0] != 0 || row_ptr[n] != m)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "row_ptr must start at 0 and end at num_edges");
  for (int i = 0; i < n; ++i)
    if (row_ptr[i + 1] < row_ptr[i]) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "row_ptr not monotone");
  for (int64_t k = 0; k < m; ++k)
    if (col_ind[k] >= n) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "col_ind out of range");
  if (!(cfg.delta > 0.0f)) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "delta must be positive");
  int lanes = cfg.narrow_lanes == 0 ? 8 : cfg.narrow_lanes;
  if (lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "narrow_lanes must be 4, 8, 16 or 32");
  DLP_CUDA_TRY(cudaSetDevice(cfg.device));
  DLP_TRY(dlp::require_device());

  dlp_session *s = new dlp_session();
  s->device = cfg.device;
  s->cfg = cfg;
  s->n = n;
  s->m = m;
  s->lanes = lanes;
  s->kernel = dlp::session::batch_kernel_ptr(lanes);
  auto bail = [&](int status) {
    delete s;
    return status;
  };
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(dlp::fail(DLP_ERR_CUDA, "stream creation failed"));
  for (int i = 0; i < kStatsRing; ++i) {
    cudaEventCreate(&s->ev[i][0]);
    cudaEventCreate(&s->ev[i][1]);
  }
  s->ev_made = true;

  // Persistent grid: as many blocks as can be co-resident.
  int dev_sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, cfg.device);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, s->kernel, dlp::session::kBlock, 0) != cudaSuccess ||
      per_sm <= 0)
    return bail(dlp::fail(DLP_ERR_CUDA, "occupancy query failed for the batch kernel"));
  if (cfg.blocks_per_sm > 0) per_sm = std::min(per_sm, cfg.blocks_per_sm);
  s->grid = dev_sms * per_sm;

  // Auto tau: mean full-graph weight (src/dynLP.cu:186-190).
  s->tau = cfg.tau < 0.0f ? dlp_mean_edge_weight(m, col_ind, values) : cfg.tau;

  DevState &d = s->st;
  d.n = n;
  int *col_tmp = nullptr;
  float *val_tmp = nullptr;
  int2 *full_adj = nullptr;
  int *full_row = nullptr;
  uint8_t *truth = nullptr;
  int *bmap = nullptr;
  int st = DLP_OK;
  auto &o = s->owned;
  if ((st = dalloc(&full_row, n + 1, o)) || (st = dalloc(&full_adj, m, o)) ||
      (st = dalloc(&d.act_adj, m, o)) || (st = dalloc(&d.act_len, n, o)) ||
      (st = dalloc(&d.status, n, o)) || (st = dalloc(&d.gt, n, o)) ||
      (st = dalloc(&d.contrib, n, o)) || (st = dalloc(&d.lab0, n, o)) ||
      (st = dalloc(&d.lab1, n, o)) || (st = dalloc(&d.local, n, o)) ||
      (st = dalloc(&d.del_stamp, n, o)) || (st = dalloc(&d.gt_stamp, n, o)) ||
      (st = dalloc(&d.dirty_stamp, n, o)) || (st = dalloc(&d.front_stamp, n, o)) ||
      (st = dalloc(&d.dirty_list, n, o)) || (st = dalloc(&d.seed_list, n, o)) ||
      (st = dalloc(&d.flist, 3 * static_cast<size_t>(n), o)) ||
      (st = dalloc(&d.touched, 2 * static_cast<size_t>(n), o)) || (st = dalloc(&d.par, n, o)) ||
      (st = dalloc(&d.acc, 2 * static_cast<size_t>(n), o)) || (st = dalloc(&s->ctl, 1, o)) ||
      (st = dalloc(&s->bc, 1, o)) || (st = dalloc(&s->stats, kStatsRing, o)))
    return bail(st);
  if (true_labels && (st = dalloc(&truth, n, o))) return bail(st);
  if (vertex_batch_map && (st = dalloc(&bmap, n, o))) return bail(st);
  if (cfg.record) {
    if ((st = dalloc(&d.rec_front0, n, o)) || (st = dalloc(&d.rec_root, n, o)) ||
        (st = dalloc(&d.rec_init, n, o)) || (st = dalloc(&d.rec_fsizes, dlp::session::kRecordIters, o)) ||
        (st = dalloc(&d.rec_minid, n, o)))
      return bail(st);
  }
  d.full_row = full_row;
  d.full_adj = full_adj;
  d.truth = truth;
  d.batch_map = bmap;
  d.ctl = s->ctl;
  d.bc = s->bc;

  auto up = [&](void *dst, const void *src, size_t bytes) -> int {
    if (bytes == 0) return DLP_OK;
    DLP_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return DLP_OK;
  };
  if ((st = up(full_row, row_ptr, sizeof(int) * (n + 1)))) return bail(st);
  if (m > 0) {
    if (cudaMalloc(&col_tmp, sizeof(int) * m) != cudaSuccess ||
        cudaMalloc(&val_tmp, sizeof(float) * m) != cudaSuccess) {
      cudaFree(col_tmp);
      cudaFree(val_tmp);
      return bail(dlp::fail(DLP_ERR_OUT_OF_MEMORY, "staging of the full graph failed"));
    }
    st = up(col_tmp, col_ind, sizeof(int) * m);
    if (!st) st = up(val_tmp, values, sizeof(float) * m);
    if (!st) {
      interleave_kernel<<<1024, 256, 0, s->stream>>>(col_tmp, val_tmp, full_adj, m);
      if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s->stream) != cudaSuccess)
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
  if ((st = reset_state(s))) return bail(st);
  *out = s;
  return DLP_OK;
}

int dlp_session_destroy(dlp_session *s) {
  delete s;
  return DLP_OK;
}

int dlp_session_reset(dlp_session *s) {
  dlp::clear_error();
  if (!s) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null session");
  DLP_CUDA_TRY(cudaSetDevice(s->device));
  DLP_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return reset_state(s);
}

float dlp_session_tau(const dlp_session *s) { return s ? s->tau : 0.0f; }
void *dlp_session_stream(dlp_session *s) { return s ? static_cast<void *>(s->stream) : nullptr; }

int dlp_session_apply_batch(dlp_session *s, int batch_index, const dlp_batch_view *h,
                            dlp_batch_stats *stats) {
  dlp::clear_error();
  if (!s || !h) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  DLP_CUDA_TRY(cudaSetDevice(s->device));
  DLP_TRY(check_ids(h->inserted, h->num_inserted, s->n, "inserted"));
  DLP_TRY(check_ids(h->gt_ids, h->num_gt, s->n, "gt_ids"));
  DLP_TRY(check_ids(h->deleted, h->num_deleted, s->n, "deleted"));
  DLP_TRY(check_ids(h->edge_src, h->num_edges, s->n, "edge_src"));
  DLP_TRY(check_ids(h->edge_dst, h->num_edges, s->n, "edge_dst"));
  if (h->num_gt > 0 && !h->gt_labels) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null gt_labels");
  if (h->num_edges > 0 && !h->edge_weight) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null edge_weight");
  dlp_batch_view dv;
  DLP_TRY(stage_batch(s, h, &dv));
  DLP_TRY(launch_batch(s, batch_index, &dv));
  if (stats) {
    DLP_TRY(dlp_session_synchronize(s));
    return dlp_session_stats(s, batch_index, stats);
  }
  return DLP_OK;
}

int dlp_session_apply_batch_device(dlp_session *s, int batch_index, const dlp_batch_view *dv) {
  dlp::clear_error();
  if (!s || !dv) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  DLP_CUDA_TRY(cudaSetDevice(s->device));
  return launch_batch(s, batch_index, dv);
}

int dlp_session_synchronize(dlp_session *s) {
  dlp::clear_error();
  if (!s) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null session");
  DLP_CUDA_TRY(cudaSetDevice(s->device));
  DLP_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return device_error(s);
}

int dlp_session_stats(dlp_session *s, int batch_index, dlp_batch_stats *out) {
  dlp::clear_error();
  if (!s || !out) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  int seq = -1;
  for (int q = static_cast<int>(s->seq_batch.size()) - 1; q >= 0; --q)
    if (s->seq_batch[q] == batch_index) {
      seq = q;
      break;
    }
  if (seq < 0 || s->seq - seq > kStatsRing)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "no statistics kept for that batch");
  DLP_CUDA_TRY(cudaSetDevice(s->device));
  DLP_CUDA_TRY(cudaStreamSynchronize(s->stream));
  DLP_TRY(device_error(s));
  const int slot = seq % kStatsRing;
  DLP_CUDA_TRY(cudaMemcpy(out, s->stats + slot, sizeof(*out), cudaMemcpyDeviceToHost));
  float ms = 0.0f;
  if (cudaEventElapsedTime(&ms, s->ev[slot][0], s->ev[slot][1]) == cudaSuccess) out->device_ms = ms;
  else cudaGetLastError();
  return DLP_OK;
}

int dlp_session_elapsed_ms(dlp_session *s, int first, int last, float *ms) {
  dlp::clear_error();
  if (!s || !ms) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  auto find = [&](int batch) {
    for (int q = static_cast<int>(s->seq_batch.size()) - 1; q >= 0; --q)
      if (s->seq_batch[q] == batch) return q;
    return -1;
  };
  const int a = find(first), b = find(last);
  if (a < 0 || b < 0 || b < a || s->seq - a > kStatsRing)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "no events kept for that batch range");
  DLP_CUDA_TRY(cudaSetDevice(s->device));
  DLP_CUDA_TRY(cudaStreamSynchronize(s->stream));
  DLP_CUDA_TRY(cudaEventElapsedTime(ms, s->ev[a % kStatsRing][0], s->ev[b % kStatsRing][1]));
  return DLP_OK;
}

int dlp_session_read_labels(dlp_session *s, float *host_labels) {
  dlp::clear_error();
  if (!s || !host_labels) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  DLP_TRY(dlp_session_synchronize(s));
  int cb = 0;
  DLP_CUDA_TRY(cudaMemcpy(&cb, &s->ctl->cur_buf, sizeof(int), cudaMemcpyDeviceToHost));
  DLP_CUDA_TRY(cudaMemcpy(host_labels, cb ? s->st.lab1 : s->st.lab0, sizeof(float) * s->n,
                          cudaMemcpyDeviceToHost));
  return DLP_OK;
}

int dlp_session_artefact(dlp_session *s, int which, void *host_out, int64_t capacity,
                         int64_t *count) {
  dlp::clear_error();
  if (!s || !count) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  DLP_TRY(dlp_session_synchronize(s));
  const DevState &d = s->st;
  BatchCounters bc;
  DLP_CUDA_TRY(cudaMemcpy(&bc, s->bc, sizeof(bc), cudaMemcpyDeviceToHost));
  dlp_batch_stats last{};
  if (s->seq > 0)
    DLP_CUDA_TRY(cudaMemcpy(&last, s->stats + (s->seq - 1) % kStatsRing, sizeof(last), cudaMemcpyDeviceToHost));
  const void *src = nullptr;
  int64_t cnt = 0;
  std::vector<float> labels;
  switch (which) {
    case DLP_ART_SEED_MARKS: src = d.seed_list; cnt = bc.num_seeds; break;
    case DLP_ART_FRONTIER0:
      if (!s->cfg.record) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "session was not created with record");
      src = d.rec_front0; cnt = bc.seed_frontier; break;
    case DLP_ART_SUB_EDGES: {
      // kept edges are stored once as (src,dst); report both directions
      const int64_t kept = bc.num_kept;
      *count = 4 * kept;
      if (host_out && kept > 0) {
        if (capacity < 4 * kept) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "capacity too small");
        std::vector<int> pr(2 * kept);
        DLP_CUDA_TRY(cudaMemcpy(pr.data(), s->sub_pairs, sizeof(int) * 2 * kept, cudaMemcpyDeviceToHost));
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
    case DLP_ART_INIT_LABELS: {
      if (!s->cfg.record) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "session was not created with record");
      src = which == DLP_ART_COMP_ROOT ? static_cast<const void *>(d.rec_root) : d.rec_init;
      cnt = s->last_inserted;  // one entry per inserted vertex of the last batch
      break;
    }
    case DLP_ART_FRONTIER_SIZES:
      if (!s->cfg.record) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "session was not created with record");
      src = d.rec_fsizes; cnt = std::min(last.iterations, dlp::session::kRecordIters); break;
    case DLP_ART_ROW_LENGTHS: src = d.act_len; cnt = s->n; break;
    case DLP_ART_LABELS: {
      labels.resize(s->n);
      DLP_TRY(dlp_session_read_labels(s, labels.data()));
      *count = s->n;
      if (host_out) {
        if (capacity < s->n) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "capacity too small");
        std::memcpy(host_out, labels.data(), sizeof(float) * s->n);
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

}  // extern "C"
