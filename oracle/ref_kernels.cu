// Test infrastructure, not product code.
//
// Runs the reference's own per-batch path on a GPU — its runDynLP
// (src/dynLP.cu:175-587, unmodified) with its own step launchers and kernels
// (src/sparsifySubgraph.cu, src/connectedComponents.cu,
// src/labelInitialization.cu, src/iterativePropagation.cu) built with its own
// flags (-O3 --use_fast_math) — on inputs from its own generator
// (src/generateSparseGraph.cu, src/generateBatches.cu), and records what each
// step produced, batch by batch, so the tests can compare the CPU oracle with
// the reference's kernels rather than with a restatement of them.
//
// Built by oracle/Makefile (target `refkern`) from the guarded copy in
// oracle/_ref/src (oracle/guard_reference.py: three index -1 accesses of the
// components step guarded). The launchers' definitions are compiled under
// other names (-DlaunchX=ref_launchX); this file defines launchX, which
// runDynLP calls, as a pass-through that also records the step's outputs:
//   launchBuildSparsifiedSubgraph  numNewEdges, numSubEdges, tau
//   launchConnectedComponents      numComponents, component id per inserted vertex
//   launchLabelInitialization      label per inserted vertex after the step
//   launchIterativePropagation     its inputs (active CSR, labels, status,
//                                  ground-truth classes, affected flags),
//                                  iterationsUsed, labels on exit
// One pass-through changes an argument: the components step is given
// min(numSubEdges, numNewEdges) edges, because the reference reads
// numSubEdges entries of an edge list of numNewEdges (src/dynLP.cu:437-440)
// and numSubEdges can be larger; the oracle pins the same bound.
//
// usage: ref_kernels n avgDegree numBatches seed maxIter out.bin [record]
// Without `record` nothing is copied back inside the batches, so the batch
// times runDynLP reports are those of the reference's path as shipped.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "dynLP.h"
#include "generateBatches.h"
#include "generateSparseGraph.h"
#include "graphTypes.h"

// The reference's launchers under their build-time names.
void ref_launchMarkDeletions(int *d_rowPtr, int *d_colInd, int *d_vertexStatus, int *d_isAffected,
                             const int *d_deletedNodes, int numDeleted, int numNodes, cudaStream_t stream);
void ref_launchBuildSparsifiedSubgraph(int *d_rowPtr, int *d_colInd, float *d_values, int *d_isAffected,
                                       const int *d_vertexStatus, const int *d_newEdgeSrc, const int *d_newEdgeDst,
                                       const float *d_newEdgeWeight, int numNewEdges, const int *d_insertedNodes,
                                       int numInserted, const int *d_isNewVertex, float tau, int *d_subRowPtr,
                                       int *d_subColInd, float *d_subValues, int &numSubNodes, int &numSubEdges,
                                       cudaStream_t stream);
void ref_launchConnectedComponents(const int *d_edgeSrc, const int *d_edgeDst, int numEdges,
                                   const int *d_insertedNodes, int numInserted, int *d_componentId,
                                   int &numComponents, int numNodes, cudaStream_t stream);
void ref_launchLabelInitialization(const int *d_rowPtr, const int *d_colInd, const float *d_values,
                                   float *d_labels, const int *d_vertexStatus, const int *d_componentId,
                                   int numComponents, const int *d_insertedNodes, int numInserted,
                                   const int *d_gtClass, int numNodes, cudaStream_t stream);
void ref_launchIterativePropagation(const int *d_rowPtr, const int *d_colInd, const float *d_values,
                                    float *d_labels, float *d_labelsBuffer, const int *d_vertexStatus,
                                    const int *d_gtClass, int *d_isAffected, int numNodes, float delta,
                                    int maxIterations, int &iterationsUsed, cudaStream_t stream);

namespace {

// What one batch's steps produced.
struct BatchRecord {
  int num_new_edges = -1;   // -1: the sparsify step did not run
  int num_sub_edges = 0;
  int hook_edges = -1;      // -1: the components step did not run
  int num_components = -1;
  int iterations = 0;
  std::vector<int> comp_id;       // per inserted position
  std::vector<float> init_labels; // per inserted position (-1 entries absent: step did not run)
  std::vector<int> seed_marks;    // vertices flagged affected when propagation starts
  std::vector<float> labels;      // all vertices after propagation
  // everything propagation starts from (its launcher's inputs), so that
  // another propagation can be run from exactly the same state
  std::vector<int> in_row_ptr, in_col_ind, in_status, in_gt, in_affected;
  std::vector<float> in_values, in_labels;
};

bool g_record = false;
float g_tau = 0.0f;
int g_num_new_edges = 0;
BatchRecord g_cur;
std::vector<BatchRecord> g_batches;

void check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    fprintf(stderr, "ref_kernels: %s: %s\n", what, cudaGetErrorString(e));
    exit(3);
  }
}

template <class T>
std::vector<T> fetch(const T *d, size_t count, cudaStream_t s) {
  std::vector<T> h(count);
  check(cudaStreamSynchronize(s), "stream sync");
  if (count) check(cudaMemcpy(h.data(), d, count * sizeof(T), cudaMemcpyDeviceToHost), "copy back");
  return h;
}

void put_i64(FILE *f, int64_t v) { fwrite(&v, sizeof(v), 1, f); }

template <class T>
void put_vec(FILE *f, const std::vector<T> &v) {
  put_i64(f, static_cast<int64_t>(v.size()));
  if (!v.empty()) fwrite(v.data(), sizeof(T), v.size(), f);
}

}  // namespace

void launchMarkDeletions(int *d_rowPtr, int *d_colInd, int *d_vertexStatus, int *d_isAffected,
                         const int *d_deletedNodes, int numDeleted, int numNodes, cudaStream_t stream) {
  ref_launchMarkDeletions(d_rowPtr, d_colInd, d_vertexStatus, d_isAffected, d_deletedNodes, numDeleted, numNodes,
                          stream);
}

void launchBuildSparsifiedSubgraph(int *d_rowPtr, int *d_colInd, float *d_values, int *d_isAffected,
                                   const int *d_vertexStatus, const int *d_newEdgeSrc, const int *d_newEdgeDst,
                                   const float *d_newEdgeWeight, int numNewEdges, const int *d_insertedNodes,
                                   int numInserted, const int *d_isNewVertex, float tau, int *d_subRowPtr,
                                   int *d_subColInd, float *d_subValues, int &numSubNodes, int &numSubEdges,
                                   cudaStream_t stream) {
  ref_launchBuildSparsifiedSubgraph(d_rowPtr, d_colInd, d_values, d_isAffected, d_vertexStatus, d_newEdgeSrc,
                                    d_newEdgeDst, d_newEdgeWeight, numNewEdges, d_insertedNodes, numInserted,
                                    d_isNewVertex, tau, d_subRowPtr, d_subColInd, d_subValues, numSubNodes,
                                    numSubEdges, stream);
  g_tau = tau;
  g_num_new_edges = numNewEdges;
  g_cur.num_new_edges = numNewEdges;
  g_cur.num_sub_edges = numSubEdges;
}

void launchConnectedComponents(const int *d_edgeSrc, const int *d_edgeDst, int numEdges, const int *d_insertedNodes,
                               int numInserted, int *d_componentId, int &numComponents, int numNodes,
                               cudaStream_t stream) {
  const int hooked = std::min(numEdges, g_num_new_edges);
  ref_launchConnectedComponents(d_edgeSrc, d_edgeDst, hooked, d_insertedNodes, numInserted, d_componentId,
                                numComponents, numNodes, stream);
  g_cur.hook_edges = hooked;
  g_cur.num_components = numComponents;
  if (g_record) {
    const std::vector<int> ins = fetch(d_insertedNodes, numInserted, stream);
    const std::vector<int> comp = fetch(d_componentId, numNodes, stream);
    g_cur.comp_id.resize(numInserted);
    for (int i = 0; i < numInserted; ++i) g_cur.comp_id[i] = comp[ins[i]];
  }
}

void launchLabelInitialization(const int *d_rowPtr, const int *d_colInd, const float *d_values, float *d_labels,
                               const int *d_vertexStatus, const int *d_componentId, int numComponents,
                               const int *d_insertedNodes, int numInserted, const int *d_gtClass, int numNodes,
                               cudaStream_t stream) {
  ref_launchLabelInitialization(d_rowPtr, d_colInd, d_values, d_labels, d_vertexStatus, d_componentId, numComponents,
                                d_insertedNodes, numInserted, d_gtClass, numNodes, stream);
  if (g_record) {
    const std::vector<int> ins = fetch(d_insertedNodes, numInserted, stream);
    const std::vector<float> lab = fetch(d_labels, numNodes, stream);
    g_cur.init_labels.resize(numInserted);
    for (int i = 0; i < numInserted; ++i) g_cur.init_labels[i] = lab[ins[i]];
  }
}

void launchIterativePropagation(const int *d_rowPtr, const int *d_colInd, const float *d_values, float *d_labels,
                                float *d_labelsBuffer, const int *d_vertexStatus, const int *d_gtClass,
                                int *d_isAffected, int numNodes, float delta, int maxIterations, int &iterationsUsed,
                                cudaStream_t stream) {
  if (g_record) {
    const std::vector<int> aff = fetch(d_isAffected, numNodes, stream);
    for (int v = 0; v < numNodes; ++v)
      if (aff[v]) g_cur.seed_marks.push_back(v);
    g_cur.in_row_ptr = fetch(d_rowPtr, static_cast<size_t>(numNodes) + 1, stream);
    const size_t m = static_cast<size_t>(g_cur.in_row_ptr[numNodes]);
    g_cur.in_col_ind = fetch(d_colInd, m, stream);
    g_cur.in_values = fetch(d_values, m, stream);
    g_cur.in_labels = fetch(static_cast<const float *>(d_labels), numNodes, stream);
    g_cur.in_status = fetch(d_vertexStatus, numNodes, stream);
    g_cur.in_gt = fetch(d_gtClass, numNodes, stream);
    g_cur.in_affected = aff;
  }
  ref_launchIterativePropagation(d_rowPtr, d_colInd, d_values, d_labels, d_labelsBuffer, d_vertexStatus, d_gtClass,
                                 d_isAffected, numNodes, delta, maxIterations, iterationsUsed, stream);
  g_cur.iterations = iterationsUsed;
  if (g_record) g_cur.labels = fetch(d_labels, numNodes, stream);
  g_batches.push_back(std::move(g_cur));
  g_cur = BatchRecord();
}

int main(int argc, char **argv) {
  if (argc < 7) {
    fprintf(stderr, "usage: %s n avgDegree numBatches seed maxIter out.bin [record]\n", argv[0]);
    return 2;
  }
  DynLPConfig cfg;
  cfg.totalNodes = atoi(argv[1]);
  cfg.avgDegree = atoi(argv[2]);
  cfg.numBatches = atoi(argv[3]);
  cfg.seed = static_cast<unsigned>(atoi(argv[4]));
  cfg.maxIterations = atoi(argv[5]);
  cfg.verbose = false;
  cfg.validate = false;
  const char *out = argv[6];
  g_record = argc > 7 && strcmp(argv[7], "record") == 0;

  CSRGraph g;
  std::vector<float> truth;
  if (!generateSparseGraph(cfg.totalNodes, cfg.avgDegree, cfg.seed, g, truth, "")) return 1;
  std::vector<BatchData> batches;
  if (!generateBatches(g, truth, cfg, batches)) return 1;

  std::vector<float> final_labels, times, accuracy;
  if (!runDynLP(cfg, g, truth, batches, final_labels, times, accuracy)) return 1;

  FILE *f = fopen(out, "wb");
  if (!f) return 1;
  fwrite("DLPREFK1", 1, 8, f);
  put_i64(f, cfg.totalNodes);
  put_i64(f, static_cast<int64_t>(g_batches.size()));
  put_i64(f, g_record ? 1 : 0);
  fwrite(&g_tau, sizeof(g_tau), 1, f);
  for (const BatchRecord &r : g_batches) {
    const int32_t head[5] = {r.num_new_edges, r.num_sub_edges, r.hook_edges, r.num_components, r.iterations};
    fwrite(head, sizeof(head), 1, f);
    put_vec(f, r.comp_id);
    put_vec(f, r.init_labels);
    put_vec(f, r.seed_marks);
    put_vec(f, r.labels);
    put_vec(f, r.in_row_ptr);
    put_vec(f, r.in_col_ind);
    put_vec(f, r.in_values);
    put_vec(f, r.in_labels);
    put_vec(f, r.in_status);
    put_vec(f, r.in_gt);
    put_vec(f, r.in_affected);
  }
  put_vec(f, times);
  put_vec(f, accuracy);
  put_vec(f, final_labels);
  fclose(f);
  return 0;
}
