/*
 * labelInitialization.h - drop-in for SMShovan/LabelPropCUDA
 * headers/labelInitialization.h:54-60 (calls dlp_label_initialization).
 */
#ifndef LABEL_INITIALIZATION_H
#define LABEL_INITIALIZATION_H

#include "graphTypes.h"

/* Each inserted vertex gets W_L1 / (W_L0 + W_L1) of its component (0.5 when
 * that sum is not above 1e-10 or the component is -1); ground truth gets 0/1.
 * W_Lc sums the weights of edges from the component's rows to ground-truth
 * vertices of class c, exactly (fixed point), then rounded once to fp32. */
void launchLabelInitialization(const int *d_rowPtr, const int *d_colInd, const float *d_values,
                               float *d_labels, const int *d_vertexStatus, const int *d_componentId,
                               int numComponents, const int *d_insertedNodes, int numInserted,
                               const int *d_gtClass, int numNodes, cudaStream_t stream);

#endif /* LABEL_INITIALIZATION_H */
