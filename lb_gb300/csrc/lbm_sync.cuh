// lbm_sync.cuh - shared-memory barriers, proxy fences and the device error codes of bounded waits,
// used by the row-staged step (bulk copies) and the tensor-core network (tcgen05 completions).
#pragma once

#include <stdint.h>

#include "lbm_math.cuh"

namespace lbm {

// codes left in Params::err by a CTA that gave up waiting, or by a plain-row thread whose pair is not of
// the packed kind (the row lists no longer match the classes)
enum : int { DEV_ERR_TMA_TIMEOUT = 1, DEV_ERR_MMA_TIMEOUT = 2, DEV_ERR_ROW_LIST = 3 };

constexpr int kWaitLimit = 1 << 22;  // try_wait attempts before a CTA gives up

LBM_D unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
LBM_D void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
LBM_D void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
LBM_D bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// at most kWaitLimit attempts; false when the phase did not complete
LBM_D bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
    bool ok = false;
    for (int it = 0; it < kWaitLimit && !ok; it++) ok = mbar_try_wait(bar, parity);
    return ok;
}
// order this thread's shared-memory writes before later async-proxy reads of them (bulk copies,
// tensor-core operands)
LBM_D void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

}  // namespace lbm
