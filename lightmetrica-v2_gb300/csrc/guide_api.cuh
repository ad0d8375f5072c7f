// Device-buffer entry points of the guiding network (guide.cu) for the
// guided renderer (guided.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "lmgpu.h"

namespace lmgpu {

// Raw outputs (float[40] per query) of n device queries (float[9] each).
int guide_forward_device(lmgpu_guide* g, const float* d_queries, uint64_t n, float* d_raw, cudaStream_t s);
// As guide_forward_device with the query count on the device (at most max_n).
int guide_forward_device_dn(lmgpu_guide* g, const float* d_queries, const uint32_t* d_n, uint64_t max_n,
                            float* d_raw, cudaStream_t s);

// Forward + backward of the mean loss of n device samples into the
// network's gradient; the loss is added to the network's loss word.
int guide_gradient_device(lmgpu_guide* g, const float* d_queries, const float* d_dirs, const float* d_weights,
                          uint64_t n, cudaStream_t s);

// One Adam step on the accumulated gradient (which it clears).
int guide_adam_device(lmgpu_guide* g, float lr, cudaStream_t s);

// The network's position box: lo and 1 / extent per axis.
void guide_box(const lmgpu_guide* g, float lo[3], float inv_ext[3]);

// Reads (and clears) the loss word and the status word; LMGPU_ERR_OVERFLOW if
// a tensor-core wait timed out.
int guide_take_loss(lmgpu_guide* g, cudaStream_t s, float* loss);

}  // namespace lmgpu
