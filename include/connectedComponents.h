/*
 * connectedComponents.h - drop-in for SMShovan/LabelPropCUDA
 * headers/connectedComponents.h:50-54 (calls dlp_connected_components).
 */
#ifndef CONNECTED_COMPONENTS_H
#define CONNECTED_COMPONENTS_H

#include <vector>

#include "graphTypes.h"

/* Shiloach-Vishkin over the given directed edge list. Vertices that are not
 * inserted act as the reference's -1 parent: an inserted vertex connected to
 * one gets component -1. Otherwise componentId is the rank of the component's
 * smallest vertex id among all components (ascending), numComponents their
 * count; every other entry of d_componentId is -1. With numEdges == 0 every
 * entry is -1 and numComponents = numInserted, as in the reference. */
void launchConnectedComponents(const int *d_edgeSrc, const int *d_edgeDst, int numEdges,
                               const int *d_insertedNodes, int numInserted, int *d_componentId,
                               int &numComponents, int numNodes, cudaStream_t stream);

#endif /* CONNECTED_COMPONENTS_H */
