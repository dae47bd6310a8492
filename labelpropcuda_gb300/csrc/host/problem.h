// Host-side problem description: a full weighted graph, its true labels and the
// batches of vertex insertions and deletions that replay it.
//
// The layout is the one the reference's CSRGraph / BatchData carry
// (headers/graphTypes.h:90-98 and :167-182): int32 row pointers and column
// indices, fp32 weights, one row per vertex sorted by column.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace dlp {

struct HostGraph {
  int n = 0;
  std::vector<int> row_ptr{0};
  std::vector<int> col;
  std::vector<float> val;
  int64_t num_edges() const { return static_cast<int64_t>(col.size()); }
};

struct HostBatch {
  std::vector<int> inserted;
  std::vector<int> gt_ids;
  std::vector<float> gt_labels;
  std::vector<int> deleted;
  std::vector<int> edge_src;
  std::vector<int> edge_dst;
  std::vector<float> edge_w;
};

struct Problem {
  HostGraph graph;
  std::vector<float> truth;
  std::vector<HostBatch> batches;
};

// Synthetic graph with the reference generator's exact decisions
// (src/generateSparseGraph.cu:118-215): balanced shuffled labels, a spanning
// path over a random permutation, then uniform extra edges until
// n * avgDegree / 2 undirected edges, weights U(0.5,1) inside a class and
// U(0.01,0.5) across classes. Returns false on invalid sizes.
bool generate_graph(int n, int avg_degree, unsigned seed, HostGraph &g,
                    std::vector<float> &truth, std::string *err);

// Batch sequence with the reference generator's exact decisions
// (src/generateBatches.cu:44-207).
bool generate_batches(const HostGraph &g, const std::vector<float> &truth,
                      int num_batches, unsigned seed, float gt_fraction,
                      float deleted_fraction, std::vector<HostBatch> &out,
                      std::string *err);

// Writes <prefix>RowPtr.txt, ColInd.txt, Values.txt and TrueLabels.txt in the
// reference's text format (src/generateSparseGraph.cu:224-271).
bool write_csr_files(const HostGraph &g, const std::vector<float> &truth,
                     const std::string &prefix, std::string *err);

// Mean weight over all non-deleted edges, accumulated in double; 0.5 for an
// empty graph (src/dynLP.cu:90-102).
float mean_edge_weight(const HostGraph &g);

// Generator arguments that identify a problem in the binary cache. Fractions
// are kept as their float bits; `generator` is kGeneratorVersion, raised
// whenever the generator's decisions change so that older files are not used.
constexpr uint32_t kGeneratorVersion = 1;
struct ProblemKey {
  int32_t num_nodes;
  int32_t avg_degree;
  int32_t num_batches;
  uint32_t seed;
  uint32_t gt_fraction_bits;
  uint32_t deleted_fraction_bits;
  uint32_t generator;
  uint32_t reserved;
};

// File name of a key inside a cache directory.
std::string cache_file_name(const ProblemKey &key);
// Writes the problem to `path` (atomically: a temporary file, then a rename).
bool save_problem(const Problem &p, const ProblemKey &key, const std::string &path, std::string *err);
// Reads a problem written by save_problem. With `want`, a file of another key
// is refused; every file is checked against its recorded size and hash.
bool load_problem(const std::string &path, const ProblemKey *want, Problem &p, ProblemKey *key_out,
                  std::string *err);

}  // namespace dlp
