// denoiser.cuh -- the denoiser's forward pass as a stage of a simulation's
// step (ssgpu.cu); defined in denoiser.cu.
#pragma once

#include <cuda_runtime.h>

#include "../../include/ssgpu.h"

namespace ss {

// the grid shape the network was created for
void dn_shape(const ss_dn *n, int *nx, int *ny, int *np);
// y = network(x) enqueued on stream s (no synchronisation; capturable);
// returns the number of kernels launched
int dn_enqueue_forward(ss_dn *n, const float *x, float *y, cudaStream_t s);
// SS_OK, or the error a tensor-core convolution recorded (synchronises s)
int dn_status(ss_dn *n, cudaStream_t s);

}  // namespace ss
