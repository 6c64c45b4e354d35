// lbm_step_f16_comb.cu - step kernels of the combined cumulant collision for the f16 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE_COLL(StF16, 3)
}  // namespace lbm
