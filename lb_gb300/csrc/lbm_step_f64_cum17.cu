// lbm_step_f64_cum17.cu - step kernels of the cumulant-2017 collision for the f64 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE_COLL(StF64, 2)
}  // namespace lbm
