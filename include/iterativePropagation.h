/*
 * iterativePropagation.h - drop-in for SMShovan/LabelPropCUDA
 * headers/iterativePropagation.h:73-80 (calls dlp_iterative_propagation).
 */
#ifndef ITERATIVE_PROPAGATION_H
#define ITERATIVE_PROPAGATION_H

#include "graphTypes.h"

/* Frontier propagation with the reference's two-buffer schedule: pass k reads
 * one buffer and writes the other at frontier vertices only; the frontier of
 * pass k+1 is the non-deleted, non-ground-truth neighbours of vertices whose
 * label moved by more than delta, plus those vertices. The whole loop runs on
 * the device; iterationsUsed is the number of passes. On return d_labels holds
 * the final labels (ground truth forced to 0/1) and d_isAffected the last
 * pass's marks. */
void launchIterativePropagation(const int *d_rowPtr, const int *d_colInd, const float *d_values,
                                float *d_labels, float *d_labelsBuffer, const int *d_vertexStatus,
                                const int *d_gtClass, int *d_isAffected, int numNodes, float delta,
                                int maxIterations, int &iterationsUsed, cudaStream_t stream);

#endif /* ITERATIVE_PROPAGATION_H */
