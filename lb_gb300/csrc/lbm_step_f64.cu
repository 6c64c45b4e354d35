// lbm_step_f64.cu - kernels instantiated for the f64 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE(StF64)
}  // namespace lbm
