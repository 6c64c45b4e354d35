// lbm_step_f64_cum15.cu - step kernels of the cumulant-2015 collision for the f64 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE_COLL(StF64, 1)
}  // namespace lbm
