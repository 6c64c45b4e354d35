// lbm_step_f32_cum15.cu - step kernels of the cumulant-2015 collision for the f32 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE_COLL(StF32, 1)
}  // namespace lbm
