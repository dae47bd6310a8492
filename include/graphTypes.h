/*
 * graphTypes.h - data types shared with code written against
 * SMShovan/LabelPropCUDA (headers/graphTypes.h there).
 *
 * Names, member order, member types and defaults are kept identical so that
 * a translation unit compiled against the reference's header links against
 * this library unchanged. CUDA_CHECK / CUDA_KERNEL_CHECK keep their
 * print-and-exit behaviour for such callers; the library itself reports
 * errors through dlp_gb300.h status codes and never exits.
 */
#ifndef GRAPH_TYPES_H
#define GRAPH_TYPES_H

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#define CUDA_CHECK(call)                                                        \
  do {                                                                          \
    cudaError_t err_ = (call);                                                  \
    if (err_ != cudaSuccess) {                                                  \
      fprintf(stderr, "CUDA Error at %s:%d - %s\n", __FILE__, __LINE__,        \
              cudaGetErrorString(err_));                                        \
      exit(EXIT_FAILURE);                                                       \
    }                                                                           \
  } while (0)

#define CUDA_KERNEL_CHECK()                                                     \
  do {                                                                          \
    cudaError_t err_ = cudaGetLastError();                                      \
    if (err_ != cudaSuccess) {                                                  \
      fprintf(stderr, "CUDA Kernel Error at %s:%d - %s\n", __FILE__, __LINE__, \
              cudaGetErrorString(err_));                                        \
      exit(EXIT_FAILURE);                                                       \
    }                                                                           \
  } while (0)

/* Host CSR: rowPtr has numNodes+1 entries; a soft-deleted entry has colInd -1. */
struct CSRGraph {
  std::vector<int> rowPtr;
  std::vector<int> colInd;
  std::vector<float> values;
  int numNodes;
  int numEdges;

  CSRGraph() : numNodes(0), numEdges(0) { rowPtr.push_back(0); }
};

/* Raw device pointers of a CSR (declared by the reference, unused by its code). */
struct DeviceCSR {
  int *d_rowPtr;
  int *d_colInd;
  float *d_values;
  int numNodes;
  int numEdges;
};

/* Run configuration; defaults as in the reference (headers/graphTypes.h:147-153). */
struct DynLPConfig {
  int totalNodes;
  int avgDegree;
  int numBatches;
  unsigned int seed;

  float tau;             /* < 0: mean edge weight of the full graph */
  float delta;
  int maxIterations;

  float groundTruthFraction;
  float unlabeledFraction;
  float deletedFraction;

  std::string outputDir;
  bool validate;
  bool verbose;

  DynLPConfig()
      : totalNodes(50000), avgDegree(5), numBatches(10), seed(42), tau(-1.0f), delta(0.0001f),
        maxIterations(100000), groundTruthFraction(0.01f), unlabeledFraction(0.90f),
        deletedFraction(0.09f), outputDir("output/"), validate(true), verbose(true) {}
};

/* One batch: inserted vertices (some with ground truth), deleted vertices and
 * the edges that become live with this batch. */
struct BatchData {
  std::vector<int> insertedNodeIds;
  std::vector<int> groundTruthNodeIds;
  std::vector<float> groundTruthLabels;
  std::vector<int> deletedNodeIds;
  std::vector<int> newEdgeSrc;
  std::vector<int> newEdgeDst;
  std::vector<float> newEdgeWeight;
  int batchId;
};

enum VertexStatus : int {
  VERTEX_ACTIVE = 0,
  VERTEX_DELETED = 1,
  VERTEX_GROUND_TRUTH = 2
};

#endif /* GRAPH_TYPES_H */
