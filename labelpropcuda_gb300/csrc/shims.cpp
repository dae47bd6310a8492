// C++ entry points with the reference's exact names and signatures
// (SMShovan/LabelPropCUDA headers/*.h), implemented over the C ABI. A program
// written against the reference (its src/main.cu included) compiles against
// include/ and links against libdynlp_gb300.so unchanged.
//
// Error behaviour follows the reference: the launchers print the failure and
// exit (its CUDA_CHECK does the same); the host functions return false.

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "connectedComponents.h"
#include "dlp_gb300.h"
#include "dynLP.h"
#include "generateBatches.h"
#include "generateSparseGraph.h"
#include "host/problem.h"
#include "iterativePropagation.h"
#include "labelInitialization.h"
#include "sparsifySubgraph.h"
#include "utils.h"
#include "validation.h"

namespace {

void die_on(int status, const char *where) {
  if (status == DLP_OK) return;
  fprintf(stderr, "DynLP error in %s: %s (%s)\n", where, dlp_status_string(status), dlp_last_error());
  exit(EXIT_FAILURE);
}

}  // namespace

// ------------------------------------------------------------ launchers ----

void launchMarkDeletions(int *d_rowPtr, int *d_colInd, int *d_vertexStatus, int *d_isAffected,
                         const int *d_deletedNodes, int numDeleted, int numNodes, cudaStream_t stream) {
  die_on(dlp_mark_deletions(d_rowPtr, d_colInd, d_vertexStatus, d_isAffected, d_deletedNodes, numDeleted,
                            numNodes, stream),
         "launchMarkDeletions");
}

void launchBuildSparsifiedSubgraph(int *d_rowPtr, int *d_colInd, float *d_values, int *d_isAffected,
                                   const int *d_vertexStatus, const int *d_newEdgeSrc, const int *d_newEdgeDst,
                                   const float *d_newEdgeWeight, int numNewEdges, const int *d_insertedNodes,
                                   int numInserted, const int *d_isNewVertex, float tau, int *d_subRowPtr,
                                   int *d_subColInd, float *d_subValues, int &numSubNodes, int &numSubEdges,
                                   cudaStream_t stream) {
  die_on(dlp_build_sparsified_subgraph(d_rowPtr, d_colInd, d_values, d_isAffected, d_vertexStatus, d_newEdgeSrc,
                                       d_newEdgeDst, d_newEdgeWeight, numNewEdges, d_insertedNodes, numInserted,
                                       d_isNewVertex, tau, d_subRowPtr, d_subColInd, d_subValues, &numSubNodes,
                                       &numSubEdges, stream),
         "launchBuildSparsifiedSubgraph");
}

void launchConnectedComponents(const int *d_edgeSrc, const int *d_edgeDst, int numEdges,
                               const int *d_insertedNodes, int numInserted, int *d_componentId,
                               int &numComponents, int numNodes, cudaStream_t stream) {
  die_on(dlp_connected_components(d_edgeSrc, d_edgeDst, numEdges, d_insertedNodes, numInserted, d_componentId,
                                  &numComponents, numNodes, stream),
         "launchConnectedComponents");
}

void launchLabelInitialization(const int *d_rowPtr, const int *d_colInd, const float *d_values, float *d_labels,
                               const int *d_vertexStatus, const int *d_componentId, int numComponents,
                               const int *d_insertedNodes, int numInserted, const int *d_gtClass, int numNodes,
                               cudaStream_t stream) {
  die_on(dlp_label_initialization(d_rowPtr, d_colInd, d_values, d_labels, d_vertexStatus, d_componentId,
                                  numComponents, d_insertedNodes, numInserted, d_gtClass, numNodes, stream),
         "launchLabelInitialization");
}

void launchIterativePropagation(const int *d_rowPtr, const int *d_colInd, const float *d_values, float *d_labels,
                                float *d_labelsBuffer, const int *d_vertexStatus, const int *d_gtClass,
                                int *d_isAffected, int numNodes, float delta, int maxIterations,
                                int &iterationsUsed, cudaStream_t stream) {
  die_on(dlp_iterative_propagation(d_rowPtr, d_colInd, d_values, d_labels, d_labelsBuffer, d_vertexStatus,
                                   d_gtClass, d_isAffected, numNodes, delta, maxIterations, &iterationsUsed,
                                   stream),
         "launchIterativePropagation");
}

void launchIrLP(const int *d_rowPtr, const int *d_colInd, const float *d_values, float *d_labels,
                const int *d_vertexStatus, const int *d_gtClass, int numNodes, float delta, int maxIterations,
                int &iterationsUsed, cudaStream_t stream) {
  die_on(dlp_irlp(d_rowPtr, d_colInd, d_values, d_labels, d_vertexStatus, d_gtClass, numNodes, delta,
                  maxIterations, &iterationsUsed, stream),
         "launchIrLP");
}

// --------------------------------------------------------------- driver ----

bool runDynLP(const DynLPConfig &config, const CSRGraph &graph, const std::vector<float> &trueLabels,
              const std::vector<BatchData> &batches, std::vector<float> &finalLabels,
              std::vector<float> &batchTimes, std::vector<float> &batchAccuracy) {
  using std::cout;
  const int n = graph.numNodes;
  const int nb = config.numBatches;
  if (n <= 0 || static_cast<int>(batches.size()) < nb) {
    cout << "Error: runDynLP needs a graph and numBatches batches.\n";
    return false;
  }
  dlp_config cfg;
  dlp_config_default(&cfg);
  cfg.tau = config.tau;
  cfg.delta = config.delta;
  cfg.max_iterations = config.maxIterations;
  // DynLPConfig has no field for it: DLP_ARITHMETIC=reference_fast_math in the
  // environment selects the reference's fast-math division for this run
  if (const char *a = std::getenv("DLP_ARITHMETIC"))
    if (std::string(a) == "reference_fast_math") cfg.arithmetic = DLP_ARITH_REFERENCE_FAST_MATH;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cfg.device = dev;

  // vertex -> batch of arrival (src/dynLP.cu:193-198)
  std::vector<int> arrival(n, -1);
  for (int b = 0; b < nb; ++b)
    for (int v : batches[b].insertedNodeIds)
      if (v >= 0 && v < n) arrival[v] = b;

  dlp_session *s = nullptr;
  int st = dlp_session_create(&cfg, n, static_cast<int64_t>(graph.colInd.size()), graph.rowPtr.data(),
                              graph.colInd.data(), graph.values.data(),
                              trueLabels.size() >= static_cast<size_t>(n) ? trueLabels.data() : nullptr,
                              arrival.data(), &s);
  if (st != DLP_OK) {
    cout << "Error: " << dlp_status_string(st) << ": " << dlp_last_error() << "\n";
    return false;
  }
  const float tau = dlp_session_tau(s);
  if (config.tau < 0.0f) cout << "Auto tau (average edge weight): " << tau << "\n";

  batchTimes.assign(nb, 0.0f);
  batchAccuracy.assign(nb, 0.0f);
  finalLabels.assign(n, 0.5f);
  bool ok = true;
  for (int b = 0; b < nb && ok; ++b) {
    const BatchData &bd = batches[b];
    if (config.verbose) {
      cout << "--- Batch " << b << " ---\n";
      cout << "  Inserting " << bd.insertedNodeIds.size() << " vertices (" << bd.groundTruthNodeIds.size()
           << " GT), deleting " << bd.deletedNodeIds.size() << "\n";
    }
    dlp_batch_view v;
    v.inserted = bd.insertedNodeIds.data();
    v.num_inserted = static_cast<int>(bd.insertedNodeIds.size());
    v.gt_ids = bd.groundTruthNodeIds.data();
    v.gt_labels = bd.groundTruthLabels.data();
    v.num_gt = static_cast<int>(bd.groundTruthNodeIds.size());
    v.deleted = bd.deletedNodeIds.data();
    v.num_deleted = static_cast<int>(bd.deletedNodeIds.size());
    v.edge_src = bd.newEdgeSrc.data();
    v.edge_dst = bd.newEdgeDst.data();
    v.edge_weight = bd.newEdgeWeight.data();
    v.num_edges = static_cast<int>(bd.newEdgeSrc.size());
    dlp_batch_stats stats;
    const auto t0 = std::chrono::steady_clock::now();
    st = dlp_session_apply_batch(s, b, &v, &stats);
    const auto t1 = std::chrono::steady_clock::now();
    if (st != DLP_OK) {
      cout << "Error: batch " << b << ": " << dlp_status_string(st) << ": " << dlp_last_error() << "\n";
      ok = false;
      break;
    }
    const float ms = std::chrono::duration<float, std::milli>(t1 - t0).count();
    batchTimes[b] = ms;
    batchAccuracy[b] = stats.accuracy;
    if (config.verbose) {
      if (stats.init_branch == 1) {
        cout << "  Step 1: " << stats.num_components << " connected components, " << stats.num_sub_edges
             << " subgraph edges (tau=" << tau << ")\n";
        cout << "  Step 2: Labels initialized for " << bd.insertedNodeIds.size() << " new vertices\n";
      }
      cout << "  Step 3: Converged in " << stats.iterations << " iterations\n";
      cout << "  Accuracy: " << (stats.accuracy * 100.0f) << "%, Time: " << ms << " ms\n\n";
    }
  }
  if (ok && dlp_session_read_labels(s, finalLabels.data()) != DLP_OK) {
    cout << "Error: " << dlp_last_error() << "\n";
    ok = false;
  }
  dlp_session_destroy(s);
  return ok;
}

// ----------------------------------------------------------- generators ----

bool generateSparseGraph(int totalNodes, int avgDegree, unsigned int seed, CSRGraph &graph,
                         std::vector<float> &trueLabels, const std::string &outputPrefix) {
  dlp::HostGraph g;
  std::string err;
  if (!dlp::generate_graph(totalNodes, avgDegree, seed, g, trueLabels, &err)) {
    std::cout << "Error: " << err << ".\n";
    return false;
  }
  std::cout << "Generated graph: " << totalNodes << " nodes, " << g.num_edges() / 2
            << " undirected edges (avg degree ~" << (static_cast<double>(g.num_edges()) / totalNodes) << ")\n";
  graph.numNodes = g.n;
  graph.numEdges = static_cast<int>(g.num_edges());
  graph.rowPtr = std::move(g.row_ptr);
  graph.colInd = std::move(g.col);
  graph.values = std::move(g.val);
  if (!outputPrefix.empty()) {
    const size_t slash = outputPrefix.find_last_of('/');
    if (!ensureDirectory(outputPrefix.substr(0, slash))) return false;
    dlp::HostGraph view;
    view.n = graph.numNodes;
    view.row_ptr = graph.rowPtr;
    view.col = graph.colInd;
    view.val = graph.values;
    if (!dlp::write_csr_files(view, trueLabels, outputPrefix, &err)) {
      std::cout << "Error: " << err << ".\n";
      return false;
    }
    std::cout << "CSR graph written to: " << outputPrefix << "*.txt\n";
  }
  return true;
}

bool generateBatches(const CSRGraph &graph, const std::vector<float> &trueLabels, const DynLPConfig &config,
                     std::vector<BatchData> &batches) {
  dlp::HostGraph g;
  g.n = graph.numNodes;
  g.row_ptr = graph.rowPtr;
  g.col = graph.colInd;
  g.val = graph.values;
  std::vector<dlp::HostBatch> hb;
  std::string err;
  if (!dlp::generate_batches(g, trueLabels, config.numBatches, config.seed, config.groundTruthFraction,
                             config.deletedFraction, hb, &err)) {
    std::cout << "Error: " << err << ".\n";
    return false;
  }
  batches.assign(hb.size(), BatchData{});
  for (size_t b = 0; b < hb.size(); ++b) {
    BatchData &d = batches[b];
    d.batchId = static_cast<int>(b);
    d.insertedNodeIds = std::move(hb[b].inserted);
    d.groundTruthNodeIds = std::move(hb[b].gt_ids);
    d.groundTruthLabels = std::move(hb[b].gt_labels);
    d.deletedNodeIds = std::move(hb[b].deleted);
    d.newEdgeSrc = std::move(hb[b].edge_src);
    d.newEdgeDst = std::move(hb[b].edge_dst);
    d.newEdgeWeight = std::move(hb[b].edge_w);
  }
  std::cout << "\nBatch generation summary:\n";
  for (size_t b = 0; b < batches.size(); ++b)
    std::cout << "  Batch " << b << ": " << batches[b].insertedNodeIds.size() << " inserted ("
              << batches[b].groundTruthNodeIds.size() << " GT), " << batches[b].deletedNodeIds.size()
              << " deleted, " << batches[b].newEdgeSrc.size() << " edges\n";
  std::cout << "\n";
  return true;
}

// --------------------------------------------------------- CLI and files ----

bool parseArguments(int argc, char *argv[], DynLPConfig &config) {
  using std::cout;
  for (int i = 1; i < argc; ++i) {
    const std::string arg = argv[i];
    const bool has_value = i + 1 < argc;
    if (arg == "--totalNodes" && has_value) {
      config.totalNodes = atoi(argv[++i]);
      if (config.totalNodes <= 0) { cout << "Error: --totalNodes must be positive.\n"; return false; }
    } else if (arg == "--numBatches" && has_value) {
      config.numBatches = atoi(argv[++i]);
      if (config.numBatches <= 0) { cout << "Error: --numBatches must be positive.\n"; return false; }
    } else if (arg == "--avgDegree" && has_value) {
      config.avgDegree = atoi(argv[++i]);
      if (config.avgDegree <= 0) { cout << "Error: --avgDegree must be positive.\n"; return false; }
    } else if (arg == "--tau" && has_value) {
      config.tau = static_cast<float>(atof(argv[++i]));
    } else if (arg == "--delta" && has_value) {
      config.delta = static_cast<float>(atof(argv[++i]));
      if (config.delta <= 0.0f) { cout << "Error: --delta must be positive.\n"; return false; }
    } else if (arg == "--maxIter" && has_value) {
      config.maxIterations = atoi(argv[++i]);
    } else if (arg == "--gtFraction" && has_value) {
      config.groundTruthFraction = static_cast<float>(atof(argv[++i]));
      if (config.groundTruthFraction <= 0.0f || config.groundTruthFraction >= 1.0f) {
        cout << "Error: --gtFraction must be in (0, 1).\n";
        return false;
      }
    } else if (arg == "--seed" && has_value) {
      config.seed = static_cast<unsigned int>(atoi(argv[++i]));
    } else if (arg == "--output" && has_value) {
      config.outputDir = argv[++i];
    } else if (arg == "--validate") {
      config.validate = true;
    } else if (arg == "--noValidate") {
      config.validate = false;
    } else if (arg == "--verbose") {
      config.verbose = true;
    } else if (arg == "--quiet") {
      config.verbose = false;
    } else if (arg == "--help" || arg == "-h") {
      cout << "Usage: dynLP [options]\n"
           << "\nOptions:\n"
           << "  --totalNodes N    Total vertices across all batches (default: 50000)\n"
           << "  --numBatches N    Number of dynamic batches (default: 10)\n"
           << "  --avgDegree  N    Average degree for graph gen (default: 5)\n"
           << "  --tau        F    Sparsification threshold (default: auto)\n"
           << "  --delta      F    Convergence threshold (default: 0.0001)\n"
           << "  --maxIter    N    Max propagation iterations (default: 100000)\n"
           << "  --gtFraction F    Ground-truth fraction (default: 0.01)\n"
           << "  --seed       N    RNG seed (default: 42)\n"
           << "  --output     DIR  Output directory (default: output/)\n"
           << "  --validate        Run IrLP baseline comparison\n"
           << "  --noValidate      Skip IrLP baseline\n"
           << "  --verbose         Print per-batch details\n"
           << "  --quiet           Suppress per-batch details\n"
           << "  --help, -h        Show this help message\n";
      return false;
    } else {
      cout << "Error: Unknown argument: " << arg << "\n";
      cout << "Run with --help for usage information.\n";
      return false;
    }
  }
  const float sum = config.groundTruthFraction + config.unlabeledFraction + config.deletedFraction;
  if (sum > 1.001f) {
    cout << "Error: Batch fractions (GT + unlabeled + deleted) exceed 1.0.\n";
    return false;
  }
  return true;
}

void printConfig(const DynLPConfig &c) {
  std::cout << "\n"
            << "============================================================\n"
            << " DynLP Configuration\n"
            << "============================================================\n"
            << "  Total nodes:        " << c.totalNodes << "\n"
            << "  Number of batches:  " << c.numBatches << "\n"
            << "  Average degree:     " << c.avgDegree << "\n"
            << "  Tau (sparsify):     " << (c.tau < 0 ? "auto (avg edge weight)" : std::to_string(c.tau)) << "\n"
            << "  Delta (converge):   " << c.delta << "\n"
            << "  Max iterations:     " << c.maxIterations << "\n"
            << "  GT fraction:        " << c.groundTruthFraction << "\n"
            << "  Unlabeled fraction: " << c.unlabeledFraction << "\n"
            << "  Deleted fraction:   " << c.deletedFraction << "\n"
            << "  Seed:               " << c.seed << "\n"
            << "  Output directory:   " << c.outputDir << "\n"
            << "  Validate (IrLP):    " << (c.validate ? "yes" : "no") << "\n"
            << "  Verbose:            " << (c.verbose ? "yes" : "no") << "\n"
            << "============================================================\n\n";
}

bool ensureDirectory(const std::string &dirPath) {
  namespace fs = std::filesystem;
  try {
    if (!dirPath.empty() && !fs::exists(dirPath)) fs::create_directories(dirPath);
    return true;
  } catch (const fs::filesystem_error &e) {
    std::cout << "Error: Could not create directory " << dirPath << ": " << e.what() << "\n";
    return false;
  }
}

bool writeLabelsToFile(const std::string &path, const float *labels, int numNodes) {
  const std::filesystem::path p(path);
  if (!p.parent_path().empty()) ensureDirectory(p.parent_path().string());
  std::ofstream f(path);
  if (!f.is_open()) {
    std::cout << "Error: Could not open file for writing: " << path << "\n";
    return false;
  }
  for (int i = 0; i < numNodes; ++i) f << i << " " << std::fixed << std::setprecision(6) << labels[i] << "\n";
  return true;
}

bool writeResultsCSV(const std::string &path, const float *batchTimes, const float *batchAccuracy,
                     int numBatches) {
  const std::filesystem::path p(path);
  if (!p.parent_path().empty()) ensureDirectory(p.parent_path().string());
  std::ofstream f(path);
  if (!f.is_open()) {
    std::cout << "Error: Could not open CSV file for writing: " << path << "\n";
    return false;
  }
  f << "batch,time_ms,accuracy\n";
  for (int i = 0; i < numBatches; ++i)
    f << i << "," << std::fixed << std::setprecision(2) << batchTimes[i] << "," << std::fixed
      << std::setprecision(6) << batchAccuracy[i] << "\n";
  return true;
}

// ------------------------------------------------------------------ IrLP ----

bool runIrLPValidation(const CSRGraph &activeGraph, const std::vector<int> &h_vertexStatus,
                       const std::vector<int> &h_gtClass, std::vector<float> &h_labels, int numNodes, float delta,
                       int maxIterations, int &iterationsUsed) {
  iterationsUsed = 0;
  if (numNodes <= 0 || activeGraph.numEdges <= 0) {
    std::cout << "Warning: IrLP validation skipped (empty graph).\n";
    return true;
  }
  const size_t n = static_cast<size_t>(numNodes);
  const size_t m = static_cast<size_t>(activeGraph.numEdges);
  void *rp = nullptr, *ci = nullptr, *va = nullptr, *lb = nullptr, *stt = nullptr, *gt = nullptr;
  bool ok = dlp_malloc(&rp, sizeof(int) * (n + 1)) == DLP_OK && dlp_malloc(&ci, sizeof(int) * m) == DLP_OK &&
            dlp_malloc(&va, sizeof(float) * m) == DLP_OK && dlp_malloc(&lb, sizeof(float) * n) == DLP_OK &&
            dlp_malloc(&stt, sizeof(int) * n) == DLP_OK && dlp_malloc(&gt, sizeof(int) * n) == DLP_OK;
  ok = ok && dlp_memcpy_htod(rp, activeGraph.rowPtr.data(), sizeof(int) * (n + 1)) == DLP_OK &&
       dlp_memcpy_htod(ci, activeGraph.colInd.data(), sizeof(int) * m) == DLP_OK &&
       dlp_memcpy_htod(va, activeGraph.values.data(), sizeof(float) * m) == DLP_OK &&
       dlp_memcpy_htod(lb, h_labels.data(), sizeof(float) * n) == DLP_OK &&
       dlp_memcpy_htod(stt, h_vertexStatus.data(), sizeof(int) * n) == DLP_OK &&
       dlp_memcpy_htod(gt, h_gtClass.data(), sizeof(int) * n) == DLP_OK;
  if (ok) {
    const int st = dlp_irlp(static_cast<int *>(rp), static_cast<int *>(ci), static_cast<float *>(va),
                            static_cast<float *>(lb), static_cast<int *>(stt), static_cast<int *>(gt), numNodes,
                            delta, maxIterations, &iterationsUsed, nullptr);
    ok = st == DLP_OK && dlp_memcpy_dtoh(h_labels.data(), lb, sizeof(float) * n) == DLP_OK;
  }
  if (!ok) std::cout << "Error: IrLP: " << dlp_last_error() << "\n";
  for (void *p : {rp, ci, va, lb, stt, gt})
    if (p) dlp_free(p);
  return ok;
}
