// C ABI plumbing: error reporting, device checks, the problem (input
// generation) object and small device helpers for bindings.
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>

#include <sys/stat.h>

#include "common.cuh"
#include "host/problem.h"

namespace dlp {

namespace {
thread_local std::string g_error;
}

void set_error(const std::string &msg) { g_error = msg; }
void clear_error() { g_error.clear(); }
int fail(int status, const std::string &msg) {
  g_error = msg;
  return status;
}
int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
  cudaGetLastError();  // clear a non-sticky error so the context stays usable
  g_error = std::string(what) + " failed at " + file + ":" + std::to_string(line) + ": " +
            cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? DLP_ERR_OUT_OF_MEMORY
         : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? DLP_ERR_NO_DEVICE
                                                                         : DLP_ERR_CUDA;
}

int require_device() {
  int dev = 0, count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(DLP_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
  }
  DLP_CUDA_TRY(cudaGetDevice(&dev));
  int major = 0, minor = 0;
  DLP_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  DLP_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
  if (major != 10 || minor != 3)
    return fail(DLP_ERR_NO_DEVICE, "this build targets sm_103a (GB300); device " +
                                       std::to_string(dev) + " is sm_" + std::to_string(major) +
                                       std::to_string(minor));
  return DLP_OK;
}

int launch_cooperative(const void *kernel, int grid, int block, void **args, size_t smem,
                       cudaStream_t stream) {
  DLP_CUDA_TRY(cudaLaunchCooperativeKernel(kernel, dim3(grid), dim3(block), args, smem, stream));
  return DLP_OK;
}

}  // namespace dlp

struct dlp_problem {
  dlp::Problem p;
  dlp::ProblemKey key{};  // the generator arguments (the cache key)
};

namespace {

dlp::ProblemKey problem_key(int n, int deg, int nb, unsigned seed, float gt, float del) {
  dlp::ProblemKey k{};
  k.num_nodes = n;
  k.avg_degree = deg;
  k.num_batches = nb;
  k.seed = seed;
  std::memcpy(&k.gt_fraction_bits, &gt, 4);
  std::memcpy(&k.deleted_fraction_bits, &del, 4);
  k.generator = dlp::kGeneratorVersion;
  return k;
}

}  // namespace

extern "C" {

int dlp_abi_version(void) { return DLP_ABI_VERSION; }

const char *dlp_status_string(int status) {
  switch (status) {
    case DLP_OK: return "DLP_OK";
    case DLP_ERR_INVALID_ARGUMENT: return "DLP_ERR_INVALID_ARGUMENT";
    case DLP_ERR_CUDA: return "DLP_ERR_CUDA";
    case DLP_ERR_OUT_OF_MEMORY: return "DLP_ERR_OUT_OF_MEMORY";
    case DLP_ERR_TIMEOUT: return "DLP_ERR_TIMEOUT";
    case DLP_ERR_NO_DEVICE: return "DLP_ERR_NO_DEVICE";
    case DLP_ERR_NOT_CONVERGED: return "DLP_ERR_NOT_CONVERGED";
    case DLP_ERR_INTERNAL: return "DLP_ERR_INTERNAL";
    default: return "DLP_ERR_UNKNOWN";
  }
}

const char *dlp_last_error(void) { return dlp::g_error.c_str(); }

int dlp_problem_generate(int num_nodes, int avg_degree, int num_batches, unsigned seed,
                         float gt_fraction, float deleted_fraction, dlp_problem **out) {
  dlp::clear_error();
  if (!out) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null out");
  *out = nullptr;
  if (!(gt_fraction > 0.0f && gt_fraction < 1.0f))
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "gt_fraction must be in (0, 1)");
  dlp_problem *p = new dlp_problem();
  p->key = problem_key(num_nodes, avg_degree, num_batches, seed, gt_fraction, deleted_fraction);
  std::string err;
  if (!dlp::generate_graph(num_nodes, avg_degree, seed, p->p.graph, p->p.truth, &err) ||
      !dlp::generate_batches(p->p.graph, p->p.truth, num_batches, seed, gt_fraction,
                             deleted_fraction, p->p.batches, &err)) {
    delete p;
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, err);
  }
  *out = p;
  return DLP_OK;
}

int dlp_problem_save(const dlp_problem *p, const char *path) {
  dlp::clear_error();
  if (!p || !path) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  std::string err;
  if (!dlp::save_problem(p->p, p->key, path, &err)) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, err);
  return DLP_OK;
}

int dlp_problem_load(const char *path, dlp_problem **out) {
  dlp::clear_error();
  if (!path || !out) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  dlp_problem *p = new dlp_problem();
  std::string err;
  if (!dlp::load_problem(path, nullptr, p->p, &p->key, &err)) {
    delete p;
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, err);
  }
  *out = p;
  return DLP_OK;
}

int dlp_problem_generate_cached(int num_nodes, int avg_degree, int num_batches, unsigned seed, float gt_fraction,
                                float deleted_fraction, const char *cache_dir, dlp_problem **out, int *from_cache) {
  dlp::clear_error();
  if (!out || !cache_dir || !*cache_dir) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (from_cache) *from_cache = 0;
  const dlp::ProblemKey key = problem_key(num_nodes, avg_degree, num_batches, seed, gt_fraction, deleted_fraction);
  const std::string path = std::string(cache_dir) + "/" + dlp::cache_file_name(key);
  dlp_problem *p = new dlp_problem();
  std::string err;
  if (dlp::load_problem(path, &key, p->p, &p->key, &err)) {
    *out = p;
    if (from_cache) *from_cache = 1;
    return DLP_OK;
  }
  delete p;
  // absent, stale or damaged: generate, then (re)write the file (the cache
  // directory itself is created when missing; its parent must exist)
  const int st = dlp_problem_generate(num_nodes, avg_degree, num_batches, seed, gt_fraction, deleted_fraction, out);
  if (st != DLP_OK) return st;
  if (mkdir(cache_dir, 0755) != 0 && errno != EEXIST) {
    dlp_problem_free(*out);
    *out = nullptr;
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, std::string("cannot create ") + cache_dir + ": " + std::strerror(errno));
  }
  if (!dlp::save_problem((*out)->p, key, path, &err)) {
    dlp_problem_free(*out);
    *out = nullptr;
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, err);
  }
  return DLP_OK;
}

void dlp_problem_free(dlp_problem *p) { delete p; }
int dlp_problem_num_nodes(const dlp_problem *p) { return p ? p->p.graph.n : 0; }
int64_t dlp_problem_num_edges(const dlp_problem *p) { return p ? p->p.graph.num_edges() : 0; }
int dlp_problem_num_batches(const dlp_problem *p) {
  return p ? static_cast<int>(p->p.batches.size()) : 0;
}
const int *dlp_problem_row_ptr(const dlp_problem *p) { return p ? p->p.graph.row_ptr.data() : nullptr; }
const int *dlp_problem_col_ind(const dlp_problem *p) { return p ? p->p.graph.col.data() : nullptr; }
const float *dlp_problem_values(const dlp_problem *p) { return p ? p->p.graph.val.data() : nullptr; }
const float *dlp_problem_true_labels(const dlp_problem *p) { return p ? p->p.truth.data() : nullptr; }

int dlp_problem_batch(const dlp_problem *p, int b, dlp_batch_view *out) {
  dlp::clear_error();
  if (!p || !out || b < 0 || b >= static_cast<int>(p->p.batches.size()))
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "invalid batch");
  const dlp::HostBatch &hb = p->p.batches[b];
  out->inserted = hb.inserted.data();
  out->num_inserted = static_cast<int>(hb.inserted.size());
  out->gt_ids = hb.gt_ids.data();
  out->gt_labels = hb.gt_labels.data();
  out->num_gt = static_cast<int>(hb.gt_ids.size());
  out->deleted = hb.deleted.data();
  out->num_deleted = static_cast<int>(hb.deleted.size());
  out->edge_src = hb.edge_src.data();
  out->edge_dst = hb.edge_dst.data();
  out->edge_weight = hb.edge_w.data();
  out->num_edges = static_cast<int>(hb.edge_src.size());
  return DLP_OK;
}

int dlp_problem_write_csr(const dlp_problem *p, const char *prefix) {
  dlp::clear_error();
  if (!p || !prefix) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null argument");
  std::string err;
  if (!dlp::write_csr_files(p->p.graph, p->p.truth, prefix, &err))
    return dlp::fail(DLP_ERR_INVALID_ARGUMENT, err);
  return DLP_OK;
}

float dlp_mean_edge_weight(int64_t m, const int *col, const float *val) {
  if (m <= 0 || !col || !val) return 0.5f;
  double sum = 0.0;
  int64_t count = 0;
  for (int64_t i = 0; i < m; ++i)
    if (col[i] >= 0) {
      sum += val[i];
      ++count;
    }
  return count > 0 ? static_cast<float>(sum / static_cast<double>(count)) : 0.5f;
}

int dlp_device_count(int *count) {
  dlp::clear_error();
  if (!count) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null count");
  *count = 0;
  cudaError_t e = cudaGetDeviceCount(count);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *count = 0;
  }
  return DLP_OK;
}
int dlp_device_name(int device, char *out, int capacity) {
  dlp::clear_error();
  if (!out || capacity <= 0) return dlp::fail(DLP_ERR_INVALID_ARGUMENT, "null name buffer");
  cudaDeviceProp prop;
  DLP_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
  std::snprintf(out, static_cast<size_t>(capacity), "%s sm_%d%d %d SMs", prop.name, prop.major, prop.minor,
                prop.multiProcessorCount);
  return DLP_OK;
}
int dlp_set_device(int device) {
  dlp::clear_error();
  DLP_CUDA_TRY(cudaSetDevice(device));
  return DLP_OK;
}
int dlp_malloc(void **ptr, size_t bytes) {
  dlp::clear_error();
  DLP_CUDA_TRY(cudaMalloc(ptr, bytes));
  return DLP_OK;
}
int dlp_free(void *ptr) {
  dlp::clear_error();
  DLP_CUDA_TRY(cudaFree(ptr));
  return DLP_OK;
}
int dlp_memcpy_htod(void *dst, const void *src, size_t bytes) {
  dlp::clear_error();
  DLP_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
  return DLP_OK;
}
int dlp_memcpy_dtoh(void *dst, const void *src, size_t bytes) {
  dlp::clear_error();
  DLP_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
  return DLP_OK;
}
int dlp_memset(void *ptr, int value, size_t bytes) {
  dlp::clear_error();
  DLP_CUDA_TRY(cudaMemset(ptr, value, bytes));
  return DLP_OK;
}
int dlp_device_synchronize(void) {
  dlp::clear_error();
  DLP_CUDA_TRY(cudaDeviceSynchronize());
  return DLP_OK;
}

}  // extern "C"
