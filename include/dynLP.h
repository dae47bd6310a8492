/*
 * dynLP.h - drop-in for SMShovan/LabelPropCUDA headers/dynLP.h:69-74.
 *
 * runDynLP replays every batch on the GPU through a resident dlp_session
 * (dlp_gb300.h): the whole per-batch update runs as one persistent kernel per
 * batch with no host round trip inside a batch. Outputs and their meaning are
 * the reference's: final labels of all vertices, per-batch wall time in ms
 * (host staging, transfer, kernels and the accuracy readback) and per-batch
 * accuracy of the 0.5 threshold over active non-ground-truth vertices.
 * Returns false (and prints the reason) on failure instead of exiting.
 */
#ifndef DYNLP_H
#define DYNLP_H

#include <vector>

#include "graphTypes.h"

bool runDynLP(const DynLPConfig &config, const CSRGraph &graph, const std::vector<float> &trueLabels,
              const std::vector<BatchData> &batches, std::vector<float> &finalLabels,
              std::vector<float> &batchTimes, std::vector<float> &batchAccuracy);

#endif /* DYNLP_H */
