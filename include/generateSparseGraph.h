/*
 * generateSparseGraph.h - drop-in for SMShovan/LabelPropCUDA
 * headers/generateSparseGraph.h:42 (same seeded output; writes
 * <outputPrefix>RowPtr.txt, ColInd.txt, Values.txt, TrueLabels.txt when the
 * prefix is not empty).
 */
#ifndef GENERATE_SPARSE_GRAPH_H
#define GENERATE_SPARSE_GRAPH_H

#include <string>
#include <vector>

#include "graphTypes.h"

bool generateSparseGraph(int totalNodes, int avgDegree, unsigned int seed, CSRGraph &graph,
                         std::vector<float> &trueLabels, const std::string &outputPrefix);

#endif /* GENERATE_SPARSE_GRAPH_H */
