// lbm_step_f16.cu - kernels instantiated for the f16 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE(StF16)
}  // namespace lbm
