// Continuous-batching server over a batch engine (C ABI group 2c in
// dlp_gb300.h). No counterpart in the reference, which applies one batch of
// one graph at a time from its driver loop (src/dynLP.cu:284-558).
//
// Requests (one batch for one resident graph) wait in arrival order. Each
// scheduling round admits every waiting request whose graph has no batch in
// progress and whose device bytes fit the memory budget, copies its arrays to
// a per-graph device buffer, and runs ONE sliced engine step: the admitted
// batches start (phases A-F) and every batch already in progress continues,
// all in the same launch, until the slice's propagation time is used up.
// Batches whose frontier empties end in that step and their requests
// complete; the others continue in the next round, next to whatever arrived
// meanwhile. The serial mode is the plain path: one request at a time, run to
// its end in one unsliced step.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <memory>
#include <thread>
#include <vector>

#include "engine.cuh"

namespace {

using Clock = std::chrono::steady_clock;

size_t align16(size_t x) { return (x + 15) & ~static_cast<size_t>(15); }

// Owned copy of a submitted request's arrays.
struct HostBatch {
  std::vector<int> ins, gt_ids, del, es, ed;
  std::vector<float> gt_lab, ew;

  explicit HostBatch(const dlp_batch_view &v)
      : ins(v.inserted, v.inserted + v.num_inserted),
        gt_ids(v.gt_ids, v.gt_ids + v.num_gt),
        del(v.deleted, v.deleted + v.num_deleted),
        es(v.edge_src, v.edge_src + v.num_edges),
        ed(v.edge_dst, v.edge_dst + v.num_edges),
        gt_lab(v.gt_labels, v.gt_labels + v.num_gt),
        ew(v.edge_weight, v.edge_weight + v.num_edges) {}

  dlp_batch_view view() const {
    dlp_batch_view v{};
    v.inserted = ins.data();
    v.num_inserted = static_cast<int>(ins.size());
    v.gt_ids = gt_ids.data();
    v.gt_labels = gt_lab.data();
    v.num_gt = static_cast<int>(gt_ids.size());
    v.deleted = del.data();
    v.num_deleted = static_cast<int>(del.size());
    v.edge_src = es.data();
    v.edge_dst = ed.data();
    v.edge_weight = ew.data();
    v.num_edges = static_cast<int>(es.size());
    return v;
  }
};

struct Request {
  int gid = 0;
  int batch = 0;
  dlp_batch_view host{};
  std::unique_ptr<HostBatch> owned;
  size_t batch_bytes = 0;  // the arrays on the device (in its graph's staging buffer)
  size_t bytes = 0;        // the engine's edge / deletion scratch the batch needs
  bool done = false;
  dlp_request_result res{};
};

// Per-graph device copy of its running batch (grown, reused), and the graph's
// eviction state.
struct GraphBuf {
  char *dev = nullptr;
  size_t dev_cap = 0;
  char *pinned = nullptr;
  size_t pin_cap = 0;
  int running = -1;  // request id
  bool evicted = false;
  std::vector<char> snap;  // the graph's device state while evicted
  size_t graph_bytes = 0;  // its device bytes when resident
  int nodes = 0;
  double last_use = 0.0;
  int res_edges = 0, res_deleted = 0;  // engine scratch reserved by dlp_server_reserve
};

size_t batch_bytes(const dlp_batch_view &v) {
  return align16(4 * static_cast<size_t>(v.num_inserted)) + 2 * align16(4 * static_cast<size_t>(v.num_gt)) +
         align16(4 * static_cast<size_t>(v.num_deleted)) + 3 * align16(4 * static_cast<size_t>(v.num_edges));
}

int check_request(int n, const dlp_request &r) {
  if (n <= 0) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "request for an unknown graph id");
  const dlp_batch_view &v = r.batch;
  if (v.num_inserted < 0 || v.num_gt < 0 || v.num_deleted < 0 || v.num_edges < 0)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "negative batch size");
  if ((v.num_inserted && !v.inserted) || (v.num_gt && (!v.gt_ids || !v.gt_labels)) ||
      (v.num_deleted && !v.deleted) || (v.num_edges && (!v.edge_src || !v.edge_dst || !v.edge_weight)))
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null batch array");
  auto ids_ok = [&](const int *p, int c) {
    for (int i = 0; i < c; ++i)
      if (p[i] < 0 || p[i] >= n) return false;
    return true;
  };
  if (!ids_ok(v.inserted, v.num_inserted) || !ids_ok(v.gt_ids, v.num_gt) || !ids_ok(v.deleted, v.num_deleted) ||
      !ids_ok(v.edge_src, v.num_edges) || !ids_ok(v.edge_dst, v.num_edges))
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "vertex id out of range in a request");
  return DLP_OK;
}

}  // namespace

struct dlp_server {
  dlp_engine *eng = nullptr;
  dlp_server_config cfg{};
  Clock::time_point t0;
  std::vector<Request> reqs;
  std::deque<int> queue;
  // One entry per possible graph id, sized once at creation: a reference into
  // it stays valid for the server's lifetime.
  std::vector<GraphBuf> bufs = std::vector<GraphBuf>(dlp::engine::kMaxGraphs);
  size_t running_bytes = 0;
  size_t staged_bytes = 0;  // device bytes of every graph's staging buffer
  int running = 0;
  int evictions = 0, restores = 0;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

  // gid must be a valid graph id (graph_nodes(gid) > 0).
  GraphBuf &buf(int gid) { return bufs[gid]; }

  // Graphs still evicted go back into the engine (best effort: a graph that
  // no longer fits is dropped and its id released).
  ~dlp_server() {
    for (size_t gid = 0; gid < bufs.size(); ++gid) {
      GraphBuf &b = bufs[gid];
      if (b.evicted && dlp_engine_restore_as(eng, b.snap.data(), b.snap.size(), static_cast<int>(gid)) != DLP_OK)
        dlp_engine_release_id(eng, static_cast<int>(gid));
      if (b.dev) cudaFree(b.dev);
      if (b.pinned) cudaFreeHost(b.pinned);
    }
  }

  // Vertex count of a graph resident in the engine or evicted by this server.
  int graph_nodes(int gid) {
    const int n = dlp_engine_graph_nodes(eng, gid);
    if (n > 0) return n;
    if (gid >= 0 && gid < static_cast<int>(bufs.size()) && bufs[gid].evicted) return bufs[gid].nodes;
    return -1;
  }

  void free_staging(GraphBuf &b) {
    if (b.dev) cudaFree(b.dev);
    staged_bytes -= std::min(staged_bytes, b.dev_cap);
    b.dev = nullptr;
    b.dev_cap = 0;
  }

  // Evicts graph gid: its whole device state to host memory, then its device
  // memory (graph and staging buffer) freed. Its id stays held in the engine,
  // so no other graph can take it. Only for a graph with no batch in progress.
  int evict(int gid) {
    GraphBuf &b = buf(gid);
    size_t bytes = 0;
    DLP_TRY(dlp_engine_snapshot(eng, gid, nullptr, 0, &bytes));
    b.snap.resize(bytes);
    DLP_TRY(dlp_engine_snapshot(eng, gid, b.snap.data(), bytes, &bytes));
    b.graph_bytes = dlp_engine_graph_resident_bytes(eng, gid);
    b.nodes = dlp_engine_graph_nodes(eng, gid);
    DLP_TRY(dlp_engine_remove_graph(eng, gid));
    DLP_TRY(dlp_engine_hold_id(eng, gid));
    DLP_CUDA_TRY(cudaStreamSynchronize(static_cast<cudaStream_t>(dlp_engine_stream(eng))));
    free_staging(b);
    b.evicted = true;
    ++evictions;
    return DLP_OK;
  }

  // Makes an evicted graph resident again under its id. This allocates its
  // device memory again, and its reserved engine scratch.
  int restore(int gid) {
    GraphBuf &b = buf(gid);
    DLP_TRY(dlp_engine_restore_as(eng, b.snap.data(), b.snap.size(), gid));
    b.snap.clear();
    b.snap.shrink_to_fit();
    b.evicted = false;
    ++restores;
    if (b.res_edges > 0 || b.res_deleted > 0) DLP_TRY(dlp_engine_reserve(eng, gid, b.res_edges, b.res_deleted));
    return DLP_OK;
  }

  // Bytes the budget counts: resident graphs, every staging buffer, and the
  // engine scratch of running requests.
  bool fits(size_t need) const {
    return cfg.memory_budget_bytes == 0 ||
           dlp_engine_bytes_in_use(eng) + staged_bytes + running_bytes + need <= cfg.memory_budget_bytes;
  }

  // Staging bytes a request adds to its graph's buffer.
  static size_t staging_growth(const GraphBuf &b, const Request &r) {
    const size_t total = std::max<size_t>(r.batch_bytes, 16);
    return total > b.dev_cap ? total - b.dev_cap : 0;
  }

  // Frees the staging buffers of graphs with no request running that were not
  // admitted in this round (`busy`); they are only a cache of earlier sizes.
  void free_idle_staging(const std::vector<int> &busy) {
    for (size_t g = 0; g < bufs.size(); ++g) {
      GraphBuf &b = bufs[g];
      if (!b.dev || b.running >= 0) continue;
      if (std::find(busy.begin(), busy.end(), static_cast<int>(g)) != busy.end()) continue;
      free_staging(b);
    }
  }

  // Makes room for `need()` more bytes: first the staging buffers of idle
  // graphs go, then (with evict_idle) idle resident graphs are evicted, least
  // recently used first (never `keep` nor a graph in `busy`). Sets *ok to
  // whether the bytes fit.
  template <class Need>
  int make_room(Need need, int keep, const std::vector<int> &busy, bool *ok) {
    *ok = fits(need());
    if (!*ok) {
      free_idle_staging(busy);
      *ok = fits(need());
    }
    while (!*ok && cfg.evict_idle) {
      int victim = -1;
      for (int g = 0; g < static_cast<int>(bufs.size()); ++g) {
        if (g == keep || dlp_engine_graph_nodes(eng, g) <= 0) continue;
        if (bufs[g].running >= 0) continue;
        if (std::find(busy.begin(), busy.end(), g) != busy.end()) continue;
        if (victim < 0 || bufs[g].last_use < bufs[victim].last_use) victim = g;
      }
      if (victim < 0) break;
      DLP_TRY(evict(victim));
      *ok = fits(need());
    }
    return DLP_OK;
  }

  int enqueue(const dlp_request &r, bool copy, double arrival, int *id) {
    DLP_TRY(check_request(graph_nodes(r.graph_id), r));
    Request q;
    q.gid = r.graph_id;
    q.batch = r.batch_index;
    if (copy) {
      q.owned = std::make_unique<HostBatch>(r.batch);
      q.host = q.owned->view();
    } else {
      q.host = r.batch;
    }
    q.batch_bytes = batch_bytes(q.host);
    q.bytes = 24 * static_cast<size_t>(q.host.num_edges) + 8 * static_cast<size_t>(q.host.num_deleted);
    q.res.graph_id = r.graph_id;
    q.res.batch_index = r.batch_index;
    q.res.status = DLP_OK;
    q.res.arrival_s = arrival;
    q.res.admit_s = -1.0;
    q.res.finish_s = -1.0;
    *id = static_cast<int>(reqs.size());
    reqs.push_back(std::move(q));
    queue.push_back(*id);
    return DLP_OK;
  }

  // Grows a graph's staging buffers (pinned and device) to hold `total` bytes.
  int grow(GraphBuf &b, size_t total) {
    cudaStream_t s = static_cast<cudaStream_t>(dlp_engine_stream(eng));
    if (total > b.pin_cap) {
      if (b.pinned) cudaFreeHost(b.pinned);
      b.pinned = nullptr;
      b.pin_cap = 0;
      DLP_CUDA_TRY(cudaMallocHost(&b.pinned, total * 2));
      b.pin_cap = total * 2;
    }
    if (total > b.dev_cap) {
      DLP_CUDA_TRY(cudaStreamSynchronize(s));
      free_staging(b);
      DLP_CUDA_TRY(cudaMalloc(&b.dev, total));
      b.dev_cap = total;
      staged_bytes += b.dev_cap;
    }
    return DLP_OK;
  }

  // Copies a request's arrays to its graph's device buffer (on the engine's
  // stream, ahead of the step's launch) and returns the device view.
  int stage(Request &r, GraphBuf &b, dlp_batch_view *out) {
    const size_t total = std::max<size_t>(r.batch_bytes, 16);
    cudaStream_t s = static_cast<cudaStream_t>(dlp_engine_stream(eng));
    DLP_TRY(grow(b, total));
    size_t off = 0;
    auto put = [&](const void *src, size_t bytes) {
      if (bytes) std::memcpy(b.pinned + off, src, bytes);
      const void *d = b.dev + off;
      off += align16(bytes);
      return d;
    };
    const dlp_batch_view &h = r.host;
    dlp_batch_view v{};
    v.inserted = static_cast<const int *>(put(h.inserted, 4 * static_cast<size_t>(h.num_inserted)));
    v.num_inserted = h.num_inserted;
    v.gt_ids = static_cast<const int *>(put(h.gt_ids, 4 * static_cast<size_t>(h.num_gt)));
    v.gt_labels = static_cast<const float *>(put(h.gt_labels, 4 * static_cast<size_t>(h.num_gt)));
    v.num_gt = h.num_gt;
    v.deleted = static_cast<const int *>(put(h.deleted, 4 * static_cast<size_t>(h.num_deleted)));
    v.num_deleted = h.num_deleted;
    v.edge_src = static_cast<const int *>(put(h.edge_src, 4 * static_cast<size_t>(h.num_edges)));
    v.edge_dst = static_cast<const int *>(put(h.edge_dst, 4 * static_cast<size_t>(h.num_edges)));
    v.edge_weight = static_cast<const float *>(put(h.edge_weight, 4 * static_cast<size_t>(h.num_edges)));
    v.num_edges = h.num_edges;
    if (off) DLP_CUDA_TRY(cudaMemcpyAsync(b.dev, b.pinned, off, cudaMemcpyHostToDevice, s));
    *out = v;
    return DLP_OK;
  }

  void finish(Request &r, int status, double t) {
    r.done = true;
    r.res.status = status;
    r.res.finish_s = t;
  }

  int poll(int *completed, int capacity, int *num_completed) {
    *num_completed = 0;
    const int limit = cfg.serial ? (running > 0 ? 0 : 1)
                                 : (cfg.max_batches_per_step > 0 ? cfg.max_batches_per_step
                                                                 : dlp::engine::kMaxGraphs);
    std::vector<int> gids, bidx, admitted;
    std::vector<dlp_batch_view> dv;
    std::vector<char> blocked;
    int out_n = 0;
    auto report = [&](int id) {
      if (completed && out_n < capacity) completed[out_n] = id;
      ++out_n;
    };
    const double t_admit = now();
    for (auto it = queue.begin(); it != queue.end() && static_cast<int>(gids.size()) < limit;) {
      Request &r = reqs[*it];
      if (r.gid >= static_cast<int>(blocked.size())) blocked.resize(r.gid + 1, 0);
      GraphBuf &b = buf(r.gid);  // bufs never reallocates, so b stays valid across make_room
      // one batch per graph at a time, in arrival order
      if (b.running >= 0 || blocked[r.gid]) {
        blocked[r.gid] = 1;
        ++it;
        continue;
      }
      // an evicted graph needs its own bytes back as well
      auto need = [&] { return r.bytes + staging_growth(b, r) + (b.evicted ? b.graph_bytes : 0); };
      bool ok = true;
      DLP_TRY(make_room(need, r.gid, gids, &ok));
      if (!ok) {
        if (running == 0 && gids.empty()) {  // nothing will free bytes: it can never fit
          dlp::set_error("request does not fit the memory budget");
          finish(r, DLP_ERR_OUT_OF_MEMORY, now());
          report(*it);
          it = queue.erase(it);
          continue;
        }
        blocked[r.gid] = 1;  // waits for running requests to free their bytes
        ++it;
        continue;
      }
      if (b.evicted) DLP_TRY(restore(r.gid));
      b.last_use = t_admit;
      dlp_batch_view v;
      DLP_TRY(stage(r, b, &v));
      b.running = *it;
      running_bytes += r.bytes;
      ++running;
      r.res.admit_s = t_admit;
      gids.push_back(r.gid);
      bidx.push_back(r.batch);
      dv.push_back(v);
      admitted.push_back(*it);
      it = queue.erase(it);
    }
    if (gids.empty() && running == 0) {
      *num_completed = out_n;
      return DLP_OK;
    }
    for (GraphBuf &b : bufs)
      if (b.running >= 0) ++reqs[b.running].res.steps;
    std::vector<int> fin(dlp::engine::kMaxGraphs);
    int nf = 0, nc = 0;
    const int st = dlp_engine_step_sliced(eng, static_cast<int>(gids.size()), gids.data(), bidx.data(), dv.data(),
                                          cfg.serial ? 0 : cfg.pass_budget, cfg.serial ? 0.0 : cfg.slice_us,
                                          fin.data(), &nf, &nc);
    const double t = now();
    if (st != DLP_OK) {
      // the step failed: every running request fails with it
      for (GraphBuf &b : bufs)
        if (b.running >= 0) {
          finish(reqs[b.running], st, t);
          report(b.running);
          b.running = -1;
        }
      running = 0;
      running_bytes = 0;
      *num_completed = out_n;
      return st;
    }
    for (int i = 0; i < nf; ++i) {
      GraphBuf &b = buf(fin[i]);
      if (b.running < 0) continue;
      Request &r = reqs[b.running];
      const int sst = dlp_engine_stats(eng, r.gid, r.batch, &r.res.stats);
      finish(r, sst, t);
      report(b.running);
      running_bytes -= std::min(running_bytes, r.bytes);
      --running;
      b.running = -1;
    }
    // a request the engine no longer runs can never finish: fail it rather
    // than wait for it
    int lost = 0;
    for (size_t gid = 0; gid < bufs.size(); ++gid) {
      GraphBuf &b = bufs[gid];
      if (b.running < 0 || dlp_engine_in_progress(eng, static_cast<int>(gid))) continue;
      finish(reqs[b.running], DLP_ERR_INTERNAL, t);
      report(b.running);
      running_bytes -= std::min(running_bytes, reqs[b.running].bytes);
      --running;
      b.running = -1;
      ++lost;
    }
    *num_completed = out_n;
    if (lost) return dlp::fail(DLP_ERR_INTERNAL, "the engine dropped a running batch");
    return DLP_OK;
  }
};

extern "C" {

void dlp_server_config_default(dlp_server_config *cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->slice_us = 2000.0;
}

int dlp_server_create(dlp_engine *e, const dlp_server_config *cfg, dlp_server **out) {
  dlp::clear_error();
  if (!e || !out) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  dlp_server_config c;
  if (cfg) c = *cfg;
  else dlp_server_config_default(&c);
  if (c.slice_us < 0 || c.pass_budget < 0 || c.max_batches_per_step < 0)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "negative server setting");
  dlp_server *s = new dlp_server();
  s->eng = e;
  s->cfg = c;
  s->t0 = Clock::now();
  *out = s;
  return DLP_OK;
}

int dlp_server_destroy(dlp_server *s) {
  if (s) {
    cudaStreamSynchronize(static_cast<cudaStream_t>(dlp_engine_stream(s->eng)));
    delete s;
  }
  return DLP_OK;
}

double dlp_server_clock(const dlp_server *s) { return s ? s->now() : 0.0; }

int dlp_server_reserve(dlp_server *s, int graph_id, int max_inserted, int max_gt, int max_deleted, int max_edges) {
  dlp::clear_error();
  if (!s || max_inserted < 0 || max_gt < 0 || max_deleted < 0 || max_edges < 0)
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null server or negative size");
  if (s->graph_nodes(graph_id) <= 0) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "unknown graph id");
  dlp_batch_view v{};
  v.num_inserted = max_inserted;
  v.num_gt = max_gt;
  v.num_deleted = max_deleted;
  v.num_edges = max_edges;
  const size_t total = std::max<size_t>(batch_bytes(v), 16);
  GraphBuf &b = s->buf(graph_id);
  b.res_edges = std::max(b.res_edges, max_edges);
  b.res_deleted = std::max(b.res_deleted, max_deleted);
  if (b.evicted) return DLP_OK;  // applied when the graph is restored
  DLP_TRY(s->grow(b, total));
  return dlp_engine_reserve(s->eng, graph_id, max_edges, max_deleted);
}

int dlp_server_submit(dlp_server *s, const dlp_request *req, int *request_id) {
  dlp::clear_error();
  if (!s || !req || !request_id) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  return s->enqueue(*req, true, s->now(), request_id);
}

int dlp_server_poll(dlp_server *s, int *completed_ids, int capacity, int *num_completed) {
  dlp::clear_error();
  if (!s || !num_completed) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  return s->poll(completed_ids, capacity, num_completed);
}

int dlp_server_result(const dlp_server *s, int request_id, dlp_request_result *out) {
  dlp::clear_error();
  if (!s || !out || request_id < 0 || request_id >= static_cast<int>(s->reqs.size()))
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "unknown request id");
  const Request &r = s->reqs[request_id];
  if (!r.done) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "request still pending");
  *out = r.res;
  return DLP_OK;
}

int dlp_server_evictions(const dlp_server *s, int *evictions, int *restores) {
  dlp::clear_error();
  if (!s) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null server");
  if (evictions) *evictions = s->evictions;
  if (restores) *restores = s->restores;
  return DLP_OK;
}

int dlp_server_make_resident(dlp_server *s, int graph_id) {
  dlp::clear_error();
  if (!s || s->graph_nodes(graph_id) <= 0) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "unknown graph id");
  GraphBuf &b = s->buf(graph_id);
  if (!b.evicted) return DLP_OK;
  bool ok = true;
  DLP_TRY(s->make_room([&] { return b.graph_bytes; }, graph_id, {}, &ok));
  if (!ok) return dlp::fail(DLP_ERR_OUT_OF_MEMORY, "the graph does not fit the memory budget");
  return s->restore(graph_id);
}

int dlp_server_pending(const dlp_server *s) { return s ? static_cast<int>(s->queue.size()) + s->running : 0; }

int dlp_server_replay(dlp_server *s, int count, const dlp_request *reqs, dlp_request_result *out,
                      double *makespan_s) {
  dlp::clear_error();
  if (!s || count < 0 || (count > 0 && (!reqs || !out))) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  for (int i = 1; i < count; ++i)
    if (reqs[i].arrival_s < reqs[i - 1].arrival_s)
      return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "requests must be sorted by arrival time");
  for (int i = 0; i < count; ++i) DLP_TRY(check_request(s->graph_nodes(reqs[i].graph_id), reqs[i]));
  std::vector<int> ids(count, -1);
  const double base = s->now();
  int next = 0, done = 0;
  std::vector<int> comp(dlp::engine::kMaxGraphs + 1024);
  while (done < count) {
    const double t = s->now() - base;
    while (next < count && reqs[next].arrival_s <= t) {
      DLP_TRY(s->enqueue(reqs[next], false, base + reqs[next].arrival_s, &ids[next]));
      ++next;
    }
    if (s->queue.empty() && s->running == 0) {
      if (next >= count) break;
      const double wait = reqs[next].arrival_s - (s->now() - base);
      if (wait > 0)
        std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.0002)));
      continue;
    }
    int nc = 0;
    const int st = s->poll(comp.data(), static_cast<int>(comp.size()), &nc);
    done += nc;
    if (st != DLP_OK) return st;
  }
  double last = 0.0;
  for (int i = 0; i < count; ++i) {
    dlp_request_result r = s->reqs[ids[i]].res;
    r.arrival_s -= base;
    if (r.admit_s >= 0) r.admit_s -= base;
    if (r.finish_s >= 0) r.finish_s -= base;
    last = std::max(last, r.finish_s);
    out[i] = r;
  }
  if (makespan_s) *makespan_s = last;
  return DLP_OK;
}

}  // extern "C"
