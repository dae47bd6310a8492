/*
 * sparsifySubgraph.h - drop-in for SMShovan/LabelPropCUDA
 * headers/sparsifySubgraph.h:41-43 and :78-84 (device arrays, reference
 * layout). Both call dlp_mark_deletions / dlp_build_sparsified_subgraph and,
 * like the reference's CUDA_CHECK, print and exit on failure.
 */
#ifndef SPARSIFY_SUBGRAPH_H
#define SPARSIFY_SUBGRAPH_H

#include <vector>

#include "graphTypes.h"

/* Neighbours of each deleted vertex become affected, its row is soft-deleted
 * (colInd = -1), it becomes DELETED, and entries pointing at DELETED vertices
 * are soft-deleted. */
void launchMarkDeletions(int *d_rowPtr, int *d_colInd, int *d_vertexStatus, int *d_isAffected,
                         const int *d_deletedNodes, int numDeleted, int numNodes, cudaStream_t stream);

/* numSubEdges = 2 x (new-new edges with weight > tau); endpoints of edges with
 * weight > tau whose id is below numInserted become affected. The kept edges
 * are written to d_subColInd / d_subValues (both directions, raw edge order). */
void launchBuildSparsifiedSubgraph(int *d_rowPtr, int *d_colInd, float *d_values, int *d_isAffected,
                                   const int *d_vertexStatus, const int *d_newEdgeSrc,
                                   const int *d_newEdgeDst, const float *d_newEdgeWeight, int numNewEdges,
                                   const int *d_insertedNodes, int numInserted, const int *d_isNewVertex,
                                   float tau, int *d_subRowPtr, int *d_subColInd, float *d_subValues,
                                   int &numSubNodes, int &numSubEdges, cudaStream_t stream);

#endif /* SPARSIFY_SUBGRAPH_H */
