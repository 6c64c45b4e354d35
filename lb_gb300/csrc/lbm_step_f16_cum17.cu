// lbm_step_f16_cum17.cu - step kernels of the cumulant-2017 collision for the f16 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE_COLL(StF16, 2)
}  // namespace lbm
