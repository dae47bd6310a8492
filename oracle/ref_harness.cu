// Test infrastructure, not product code.
//
// Host-only harness around the reference's own sources (SMShovan/LabelPropCUDA).
// It is compiled by oracle/Makefile (target `ref`) straight from the reference
// checkout, and its binary goes to oracle/_ref/. It never launches a kernel, so
// it runs on a machine without a GPU. It dumps what the reference's host code
// produces for a given configuration:
//   * the full graph and true labels   (src/generateSparseGraph.cu:118-215)
//   * the batches                      (src/generateBatches.cu:44-207)
//   * the auto tau                     (src/dynLP.cu:90-102, used at :186-190)
//   * the active CSR of every batch    (src/dynLP.cu:111-167, driven as at :284-309)
// tests/golden/make_golden.py turns the dump into the committed fixtures that
// pin the product's input generator and the oracle's CSR batch update.
//
// dynLP.cu keeps updateHostCSR / computeAvgEdgeWeight in an anonymous
// namespace, so this translation unit includes that source file to reach them.
#include "../src/dynLP.cu"
#include "generateBatches.h"
#include "generateSparseGraph.h"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

namespace {

void put_i64(FILE *f, int64_t v) { fwrite(&v, sizeof(v), 1, f); }

template <typename T> void put_vec(FILE *f, const std::vector<T> &v) {
  put_i64(f, static_cast<int64_t>(v.size()));
  if (!v.empty()) fwrite(v.data(), sizeof(T), v.size(), f);
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 6) {
    fprintf(stderr, "usage: %s n avgDegree numBatches seed out.bin\n", argv[0]);
    return 2;
  }
  DynLPConfig cfg;
  cfg.totalNodes = atoi(argv[1]);
  cfg.avgDegree = atoi(argv[2]);
  cfg.numBatches = atoi(argv[3]);
  cfg.seed = static_cast<unsigned>(atoi(argv[4]));
  const char *out = argv[5];

  CSRGraph g;
  std::vector<float> truth;
  if (!generateSparseGraph(cfg.totalNodes, cfg.avgDegree, cfg.seed, g, truth, "")) return 1;
  std::vector<BatchData> batches;
  if (!generateBatches(g, truth, cfg, batches)) return 1;

  FILE *f = fopen(out, "wb");
  if (!f) return 1;
  put_i64(f, g.numNodes);
  put_vec(f, g.rowPtr);
  put_vec(f, g.colInd);
  put_vec(f, g.values);
  put_vec(f, truth);
  put_i64(f, static_cast<int64_t>(batches.size()));
  for (const BatchData &b : batches) {
    put_vec(f, b.insertedNodeIds);
    put_vec(f, b.groundTruthNodeIds);
    put_vec(f, b.groundTruthLabels);
    put_vec(f, b.deletedNodeIds);
    put_vec(f, b.newEdgeSrc);
    put_vec(f, b.newEdgeDst);
    put_vec(f, b.newEdgeWeight);
  }
  float tau = computeAvgEdgeWeight(g);
  fwrite(&tau, sizeof(tau), 1, f);

  // Drive updateHostCSR exactly as runDynLP's batch loop does.
  std::vector<int> batchMap(cfg.totalNodes, -1);
  for (int b = 0; b < cfg.numBatches; ++b)
    for (int v : batches[b].insertedNodeIds) batchMap[v] = b;
  std::vector<int> status(cfg.totalNodes, VERTEX_DELETED);
  CSRGraph active;
  for (int b = 0; b < cfg.numBatches; ++b) {
    updateHostCSR(active, g, batches[b], batchMap, b, status);
    put_vec(f, active.rowPtr);
    put_vec(f, active.colInd);
    put_vec(f, active.values);
    put_vec(f, status);
  }
  fclose(f);
  return 0;
}
