/*
 * validation.h - drop-in for SMShovan/LabelPropCUDA headers/validation.h:60-88:
 * IrLP, the full-recompute baseline, on the GPU.
 */
#ifndef VALIDATION_H
#define VALIDATION_H

#include <vector>

#include "graphTypes.h"

/* Every active non-ground-truth vertex is recomputed from the previous buffer
 * each iteration, ground truth re-imposed, until no label moves by more than
 * delta. Result in d_labels. */
void launchIrLP(const int *d_rowPtr, const int *d_colInd, const float *d_values, float *d_labels,
                const int *d_vertexStatus, const int *d_gtClass, int numNodes, float delta, int maxIterations,
                int &iterationsUsed, cudaStream_t stream);

bool runIrLPValidation(const CSRGraph &activeGraph, const std::vector<int> &h_vertexStatus,
                       const std::vector<int> &h_gtClass, std::vector<float> &h_labels, int numNodes,
                       float delta, int maxIterations, int &iterationsUsed);

#endif /* VALIDATION_H */
