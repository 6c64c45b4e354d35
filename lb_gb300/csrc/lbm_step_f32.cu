// lbm_step_f32.cu - kernels instantiated for the f32 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE(StF32)
}  // namespace lbm
