// Force-included when the reference's own GPU code is compiled with CUDA 13:
// cudaGraphAddDependencies gained an edge-data argument there, and the
// reference calls the four-argument form.  This overload forwards with no
// edge data, which is what the four-argument form meant.
#pragma once
#include <cuda_runtime.h>

inline cudaError_t cudaGraphAddDependencies(cudaGraph_t graph,
                                            const cudaGraphNode_t* from,
                                            const cudaGraphNode_t* to,
                                            size_t num_dependencies) {
  return cudaGraphAddDependencies(graph, from, to, nullptr, num_dependencies);
}
