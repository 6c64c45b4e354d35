// lbm_step_f32_comb.cu - step kernels of the combined cumulant collision for the f32 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE_COLL(StF32, 3)
}  // namespace lbm
