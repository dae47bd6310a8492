/*
 * generateBatches.h - drop-in for SMShovan/LabelPropCUDA
 * headers/generateBatches.h:56 (same seeded output).
 */
#ifndef GENERATE_BATCHES_H
#define GENERATE_BATCHES_H

#include <vector>

#include "graphTypes.h"

bool generateBatches(const CSRGraph &graph, const std::vector<float> &trueLabels, const DynLPConfig &config,
                     std::vector<BatchData> &batches);

#endif /* GENERATE_BATCHES_H */
