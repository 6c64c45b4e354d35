// lbm_step_f16_cum15.cu - step kernels of the cumulant-2015 collision for the f16 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE_COLL(StF16, 1)
}  // namespace lbm
