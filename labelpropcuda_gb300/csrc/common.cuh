// Shared host and device helpers of the GB300 DynLP library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "dlp_gb300.h"

namespace dlp {

// ---------------------------------------------------------------------------
// Host-side error plumbing: every C-ABI call returns a status and leaves a
// message for the calling thread.
// ---------------------------------------------------------------------------
void set_error(const std::string &msg);
void clear_error();
int fail(int status, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define DLP_CUDA_TRY(call)                                                    \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) return ::dlp::cuda_fail(e_, #call, __FILE__, __LINE__); \
  } while (0)

#define DLP_TRY(call)                \
  do {                               \
    int s_ = (call);                 \
    if (s_ != DLP_OK) return s_;     \
  } while (0)

// Checks that a GPU of compute capability 10.3 is current.
int require_device();

// Vertex status values of the reference (headers/graphTypes.h:191-195).
constexpr int kActive = 0;
constexpr int kDeleted = 1;
constexpr int kGroundTruth = 2;

// ---------------------------------------------------------------------------
// Device primitives.
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned atom_add_acq_rel_u32(unsigned *p, unsigned v) {
  unsigned old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;"
               : "=r"(old)
               : "l"(p), "r"(v)
               : "memory");
  return old;
}
__device__ __forceinline__ int ld_relaxed_i32(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Barrier over the first `nblocks` blocks of a cooperative launch (all blocks
// co-resident). Arrivals are counted in two levels — groups of 16 blocks, then
// the groups — so they do not all serialise on one counter; the last block to
// arrive advances the generation, the others wait for it with a time limit. A
// block that runs out of time records DLP_ERR_TIMEOUT in *err and every block
// leaves at its next barrier, so no wait is unbounded.
constexpr int kBarrierGroup = 16;
constexpr int kBarrierMaxGroups = 128;

struct GridBarrier {
  unsigned count;
  unsigned gen;
  unsigned group[kBarrierMaxGroups];
};

__device__ __forceinline__ bool grid_sync_n(GridBarrier *bar, unsigned nblocks, int *err, uint64_t timeout_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned gen = ld_acquire_u32(&bar->gen);
    const unsigned ngroups = (nblocks + kBarrierGroup - 1) / kBarrierGroup;
    bool last = false;
    if (ngroups <= 1 || ngroups > kBarrierMaxGroups) {
      last = atom_add_acq_rel_u32(&bar->count, 1u) == nblocks - 1;
      if (last) bar->count = 0;
    } else {
      const unsigned grp = blockIdx.x / kBarrierGroup;
      const unsigned gsize = min(static_cast<unsigned>(kBarrierGroup), nblocks - grp * kBarrierGroup);
      if (atom_add_acq_rel_u32(&bar->group[grp], 1u) == gsize - 1) {
        bar->group[grp] = 0;  // ordered before the release of the next arrival
        last = atom_add_acq_rel_u32(&bar->count, 1u) == ngroups - 1;
        if (last) bar->count = 0;
      }
    }
    int ok = 1;
    if (last) {
      st_release_u32(&bar->gen, gen + 1);
    } else {
      const uint64_t t0 = global_timer_ns();
      unsigned spins = 0;
      while (ld_acquire_u32(&bar->gen) == gen) {
        if (((++spins) & 63u) == 0 && global_timer_ns() - t0 > timeout_ns) {
          atomicCAS(err, 0, DLP_ERR_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(20);
      }
    }
    s_ok = ok && (ld_relaxed_i32(err) == 0);
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ bool grid_sync(GridBarrier *bar, int *err, uint64_t timeout_ns) {
  return grid_sync_n(bar, gridDim.x * gridDim.y * gridDim.z, err, timeout_ns);
}

// Appends the set lanes' values to list[*count ...] with one atomic per warp.
// Must be called by all lanes of the warp (convergent).
__device__ __forceinline__ void warp_append(bool pred, int value, int *list, int *count) {
  const unsigned mask = __ballot_sync(0xffffffffu, pred);
  if (mask == 0) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(mask) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(count, __popc(mask));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (pred) list[base + __popc(mask & ((1u << lane) - 1u))] = value;
}

// Same, growing downward from list[cap - 1] (for a second list sharing the array).
__device__ __forceinline__ void warp_append_back(bool pred, int value, int *list, int cap,
                                                 int *count) {
  const unsigned mask = __ballot_sync(0xffffffffu, pred);
  if (mask == 0) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(mask) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(count, __popc(mask));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (pred) list[cap - 1 - (base + __popc(mask & ((1u << lane) - 1u)))] = value;
}

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ int warp_sum_i(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// 32.32 fixed point for exact, order-independent supernode weight sums.
__device__ __forceinline__ long long to_fixed(float w) {
  return __double2ll_rn(static_cast<double>(w) * 4294967296.0);
}
__device__ __forceinline__ float from_fixed(long long q) {
  return __double2float_rn(__ll2double_rn(q) * (1.0 / 4294967296.0));
}

// New label from the two row sums (src/iterativePropagation.cu:153-168) with an
// IEEE round-to-nearest division.
// The quotient of a weighted average. Default: IEEE round-to-nearest, the
// oracle's arithmetic. fast: the CUDA fast division (__fdividef), the division
// that the reference's -use_fast_math build makes of its `/`
// (src/iterativePropagation.cu:160, src/labelInitialization.cu:137; Makefile:52).
__device__ __forceinline__ float quotient(float num, float den, bool fast) {
  return fast ? __fdividef(num, den) : __fdiv_rn(num, den);
}

__device__ __forceinline__ float updated_label(float w_all, float w_label, float old, bool fast = false) {
  float nl = (w_all > 1e-10f) ? quotient(w_label, w_all, fast) : old;
  return fminf(fmaxf(nl, 0.0f), 1.0f);
}

// Launch helper: cooperative launch of `kernel` with `args` on `stream`.
int launch_cooperative(const void *kernel, int grid, int block, void **args, size_t smem,
                       cudaStream_t stream);

}  // namespace dlp
