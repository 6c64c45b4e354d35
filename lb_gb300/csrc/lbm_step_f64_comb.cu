// lbm_step_f64_comb.cu - step kernels of the combined cumulant collision for the f64 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE_COLL(StF64, 3)
}  // namespace lbm
