// lbm_step_f16_srt.cu - step kernels of the SRT collision for the f16 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE_COLL(StF16, 0)
}  // namespace lbm
