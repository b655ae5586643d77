// Internal interface of the learned warm-start network (tog_nn.cu) for the
// solver (tog_api.cu).
#pragma once
#include <cuda_runtime.h>

struct tog_nn;

namespace tog {
// y = network(x) on the given stream: x = nodes x 8 FP32 channels (channels-last),
// y = nodes x 3 FP32 channels
int nn_forward_dev(tog_nn* nn, const float* in_dev, float* out_dev, cudaStream_t stream);
// TOG_OK, or TOG_ERR_CUDA when a tensor-core convolution gave up waiting for its MMAs
// (synchronises the stream; the condition stays set for the network's lifetime)
int nn_status(tog_nn* nn, cudaStream_t stream);
// true when the network was created for this node grid (x, y, z node counts) and batch
bool nn_matches(const tog_nn* nn, const int nodes[3], int batch);
}  // namespace tog
