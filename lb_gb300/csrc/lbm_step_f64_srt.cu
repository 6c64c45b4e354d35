// lbm_step_f64_srt.cu - step kernels of the SRT collision for the f64 population storage.
#include "lbm_launch.cuh"

namespace lbm {
LBM_INSTANTIATE_COLL(StF64, 0)
}  // namespace lbm
