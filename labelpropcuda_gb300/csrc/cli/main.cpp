// dynlp_gb300: command-line drop-in for the reference binary bin/dynLP
// (SMShovan/LabelPropCUDA src/main.cu:53-298). Same flags, same output files
// (<output>/graph/csr*.txt, dynlp_labels.txt, results.csv, irlp_labels.txt)
// and the same summary; the per-batch path runs on the GB300 library.

#include <chrono>
#include <iomanip>
#include <iostream>
#include <numeric>
#include <vector>

#include "dynLP.h"
#include "generateBatches.h"
#include "generateSparseGraph.h"
#include "utils.h"
#include "validation.h"

int main(int argc, char *argv[]) {
  using std::cout;
  DynLPConfig config;
  if (!parseArguments(argc, argv, config)) return 1;
  printConfig(config);
  if (!ensureDirectory(config.outputDir) || !ensureDirectory(config.outputDir + "/graph")) return 1;

  cout << "Generating sparse graph...\n";
  CSRGraph full;
  std::vector<float> truth;
  if (!generateSparseGraph(config.totalNodes, config.avgDegree, config.seed, full, truth,
                           config.outputDir + "/graph/csr")) {
    cout << "Error: Graph generation failed.\n";
    return 1;
  }
  cout << "Generating batches...\n";
  std::vector<BatchData> batches;
  if (!generateBatches(full, truth, config, batches)) {
    cout << "Error: Batch generation failed.\n";
    return 1;
  }

  cout << "Running DynLP...\n\n";
  std::vector<float> labels, times, acc;
  if (!runDynLP(config, full, truth, batches, labels, times, acc)) {
    cout << "Error: DynLP execution failed.\n";
    return 1;
  }

  std::vector<float> irlp;
  float irlp_acc = 0.0f, irlp_ms = 0.0f;
  if (config.validate) {
    cout << "Running IrLP baseline for validation...\n";
    const int n = config.totalNodes;
    // Final snapshot: inserts, then deletions, then ground truth of every batch
    // in order (src/main.cu:133-147).
    std::vector<int> status(n, VERTEX_DELETED), gt(n, -1), arrival(n, -1);
    irlp.assign(n, 0.5f);
    for (int b = 0; b < config.numBatches; ++b) {
      for (int v : batches[b].insertedNodeIds) status[v] = VERTEX_ACTIVE;
      for (int v : batches[b].deletedNodeIds) status[v] = VERTEX_DELETED;
      for (size_t i = 0; i < batches[b].groundTruthNodeIds.size(); ++i) {
        const int v = batches[b].groundTruthNodeIds[i];
        status[v] = VERTEX_GROUND_TRUTH;
        gt[v] = batches[b].groundTruthLabels[i] < 0.5f ? 0 : 1;
        irlp[v] = batches[b].groundTruthLabels[i];
      }
      for (int v : batches[b].insertedNodeIds) arrival[v] = b;
    }
    CSRGraph snap;
    snap.rowPtr.assign(1, 0);
    snap.numNodes = n;
    for (int u = 0; u < n; ++u) {
      if (status[u] != VERTEX_DELETED && arrival[u] >= 0)
        for (int k = full.rowPtr[u]; k < full.rowPtr[u + 1]; ++k) {
          const int v = full.colInd[k];
          if (v < 0 || status[v] == VERTEX_DELETED || arrival[v] < 0) continue;
          snap.colInd.push_back(v);
          snap.values.push_back(full.values[k]);
        }
      snap.rowPtr.push_back(static_cast<int>(snap.colInd.size()));
    }
    snap.numEdges = static_cast<int>(snap.colInd.size());
    const auto t0 = std::chrono::steady_clock::now();
    int iters = 0;
    if (!runIrLPValidation(snap, status, gt, irlp, n, config.delta, config.maxIterations, iters)) {
      cout << "Error: IrLP validation failed.\n";
      return 1;
    }
    irlp_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    int correct = 0, total = 0;
    for (int i = 0; i < n; ++i) {
      if (status[i] == VERTEX_DELETED || status[i] == VERTEX_GROUND_TRUTH) continue;
      correct += ((irlp[i] >= 0.5f) ? 1 : 0) == ((truth[i] >= 0.5f) ? 1 : 0);
      ++total;
    }
    irlp_acc = total > 0 ? static_cast<float>(correct) / total : 1.0f;
    cout << "IrLP baseline: " << iters << " iterations, " << irlp_ms << " ms, accuracy " << std::fixed
         << std::setprecision(2) << (irlp_acc * 100.0f) << "%\n\n";
  }

  if (!writeLabelsToFile(config.outputDir + "/dynlp_labels.txt", labels.data(), config.totalNodes)) {
    cout << "Error: Could not write DynLP labels.\n";
    return 1;
  }
  if (!writeResultsCSV(config.outputDir + "/results.csv", times.data(), acc.data(), config.numBatches)) {
    cout << "Error: Could not write results CSV.\n";
    return 1;
  }
  if (config.validate && !writeLabelsToFile(config.outputDir + "/irlp_labels.txt", irlp.data(), config.totalNodes)) {
    cout << "Error: Could not write IrLP labels.\n";
    return 1;
  }

  const float total_ms = std::accumulate(times.begin(), times.end(), 0.0f);
  const float avg_acc = std::accumulate(acc.begin(), acc.end(), 0.0f) / config.numBatches;
  cout << "============================================================\n"
       << " DynLP Results Summary\n"
       << "============================================================\n"
       << "  Total DynLP time:     " << std::fixed << std::setprecision(2) << total_ms << " ms\n"
       << "  Average accuracy:     " << std::fixed << std::setprecision(2) << (avg_acc * 100.0f) << "%\n"
       << "  Final batch accuracy: " << std::fixed << std::setprecision(2) << (acc.back() * 100.0f) << "%\n";
  if (config.validate) {
    const float speedup = irlp_ms > 0.0f ? irlp_ms / total_ms : 0.0f;
    cout << "  IrLP baseline time:   " << std::fixed << std::setprecision(2) << irlp_ms << " ms\n"
         << "  IrLP accuracy:        " << std::fixed << std::setprecision(2) << (irlp_acc * 100.0f) << "%\n"
         << "  Speedup vs IrLP:      " << std::fixed << std::setprecision(1) << speedup << "x\n";
  }
  cout << "============================================================\n\nPer-batch results:\n";
  for (int b = 0; b < config.numBatches; ++b)
    cout << "  Batch " << std::setw(2) << b << ": " << std::fixed << std::setprecision(2) << std::setw(10)
         << times[b] << " ms, accuracy " << std::fixed << std::setprecision(2) << (acc[b] * 100.0f) << "%\n";
  cout << "\nOutput files written to: " << config.outputDir << "/\n"
       << "  dynlp_labels.txt  — Final predicted labels\n"
       << "  results.csv       — Per-batch timing and accuracy\n";
  if (config.validate) cout << "  irlp_labels.txt   — IrLP baseline labels\n";
  cout << "  graph/            — Generated graph in CSR format\n";
  return 0;
}
