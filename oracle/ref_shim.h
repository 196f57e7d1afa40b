/* Force-included when compiling the reference's CUDA sources (oracle/build_ref.sh).  CUDA 13 added
 * an edge-data argument to cudaGraphAddNode; the reference calls the CUDA 12 five-argument form
 * (endoscopic_tissue/native/vendor/cuda/xpbd/xpbd_solver.cu:2803).  This overload forwards it
 * with no edge data, so the reference compiles unmodified. */
#pragma once
#include <cuda_runtime_api.h>
#ifdef __cplusplus
static inline cudaError_t cudaGraphAddNode(cudaGraphNode_t* node, cudaGraph_t graph, const cudaGraphNode_t* dependencies,
                                           size_t count, struct cudaGraphNodeParams* params) {
    return cudaGraphAddNode(node, graph, dependencies, (const cudaGraphEdgeData*)0, count, params);
}
#endif
