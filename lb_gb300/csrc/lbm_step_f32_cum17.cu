// lbm_step_f32_cum17.cu - step kernels of the cumulant-2017 collision for the f32 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE_COLL(StF32, 2)
}  // namespace lbm
