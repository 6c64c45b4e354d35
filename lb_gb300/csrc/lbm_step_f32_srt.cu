// lbm_step_f32_srt.cu - step kernels of the SRT collision for the f32 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE_COLL(StF32, 0)
}  // namespace lbm
