// lbm_mlp_host.h - host-side helpers of the learned closure shared by mlp.cu and lbm_capi.cu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/lbm.h"

namespace lbm {

struct MlpNorm;

// fragment table (kMlpFragRows x 32 uint4) with the activation constants folded into FP16 weights,
// and the normalisation / range / output constants of the step kernel
void mlp_pack(const lbm_mlp_model& m, uint4* frag, MlpNorm& nm);
// finite parameters, positive scales, lo <= hi
bool mlp_model_valid(const lbm_mlp_model* m);
// box filter of width w of a fine run's moments and the per-coarse-cell samples (11 floats each:
// 7 inputs, a, b, c, valid).  cf: 11 * Nc floats of scratch, out: 11 * Nc floats.
cudaError_t launch_les_samples(const double* rho, const double* u, const uint8_t* cls, int nx, int ny, int nz, int w,
                               const int wrap[3], float* cf, float* out, cudaStream_t st);

}  // namespace lbm
