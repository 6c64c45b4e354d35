// lbm_mlp_tc.cuh - the learned closure's network on the tcgen05 tensor cores (accumulators in TMEM).
//
// A CTA of up to 128 threads evaluates the network for its cells, two per thread, as two M = 128
// tiles: row t of tile 0 is thread t's first cell, row t of tile 1 its second, so a cell's accumulator
// row sits in TMEM lane t, the lane that warp t/32 may read.  Per layer:
//   every thread stores its rows of the A operands (FP16) in shared memory and fences them for the async
//   proxy; the CTA synchronises; thread 0 issues the tcgen05.mma of both tiles (A and B from shared
//   memory, FP32 accumulators in TMEM) and commits them to an mbarrier; every thread waits on it (bounded),
//   loads its lane's accumulators with tcgen05.ld, adds the bias, applies the activation while packing to
//   FP16 (mlp_act, the same folded form as the warp path) and stores the next layer's A row.  (Alternating the two tiles, so that one
//   tile's products run while the threads work on the other's accumulators, measured slower: two more
//   CTA barriers per evaluation.)
// Shapes (kind::f16, FP16 A and B, FP32 D; H = kMlpHid hidden units): layer 1 M128 NH K16 (7 inputs, a 1
// that carries the first bias, 8 zeros); layer 2 M128 NH KH (H/16 MMAs, bias added after the load);
// layer 3 M128 N16 KH (the output in column 0; rows 1..15 of W3 are zero).  TMEM: max(2H, 32) columns per
// CTA, the accumulators of the two tiles at columns 0 and H (layer 3: 0 and 16).  Only thread 0 issues MMAs; the other threads'
// instructions are the operand stores, the TMEM loads and the pack.
// Shared-memory operands use the canonical K-major layout without swizzle: a core matrix of 8 rows x 8
// halves is 128 contiguous bytes (row r at 16 r); core matrix (row group g, k group j) of a matrix with
// KG k groups is at g * KG * 128 + j * 128, i.e. leading-dimension byte offset 128 (next k group) and
// stride-dimension byte offset KG * 128 (next group of 8 rows).
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include "lbm_mlp.cuh"
#include "lbm_sync.cuh"

namespace lbm {

// the weight image (host-packed, copied into shared memory by every CTA): W1 H x 16, W2 H x H, W3 16 x H,
// each K-major in the layout above
constexpr int kTcH = kMlpHid, kTcKG = kTcH / 8;  // hidden units; k groups of a hidden-layer operand
constexpr int kTcW1 = 0, kTcW2 = kTcH * 16 * 2, kTcW3 = kTcW2 + kTcH * kTcH * 2, kTcWBytes = kTcW3 + 16 * kTcH * 2;
constexpr int kTcWRows = kTcWBytes / 16;  // uint4 rows of the image
static_assert(kTcWRows == kMlpTcRows, "the image's size in the model buffer");
constexpr int kTcCols = 2 * kTcH < 32 ? 32 : 2 * kTcH;  // TMEM columns per CTA (a power of two >= 32)
constexpr int kTcA1Bytes = 128 * 16 * 2, kTcA2Bytes = 128 * kTcH * 2;

// byte offset of element (row, k) group: row r, k group j, in a K-major matrix with KG k groups
LBM_HD constexpr int tc_off(int row, int kg, int KG) { return (row >> 3) * KG * 128 + kg * 128 + (row & 7) * 16; }

struct __align__(128) TcSmem {
    uint4 w[kTcWRows];
    uint4 a1[2][kTcA1Bytes / 16];  // layer-1 operand of the two tiles
    uint4 a2[2][kTcA2Bytes / 16];  // layer-2 and layer-3 operands of the two tiles
    uint64_t bar;  // completion of a layer's products
    uint32_t tmem;
};

// ---- PTX ------------------------------------------------------------------------------------------------
// shared-memory matrix descriptor: start address, leading-dimension byte offset 128, stride-dimension
// byte offset `sbo`, descriptor version 1 (bits 46-47), no swizzle
LBM_D uint64_t tc_desc(const void* smem, uint32_t sbo) {
    const uint32_t a = smem_u32(smem);
    return (uint64_t)((a >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) |
           (1ull << 46);
}
// instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B FP16 (bits 7-9, 10-12 = 0), both
// K-major (bits 15, 16 = 0), N >> 3 at bit 17, M >> 4 at bit 24, M = 128
LBM_HD constexpr uint32_t tc_idesc(int n) { return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24); }

LBM_D void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
// the mbarrier completes one arrival when every tcgen05 operation this thread issued before has completed
LBM_D void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
LBM_D void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
LBM_D void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// one 32-bit column of this thread's lane; the wait is part of the same statement, so the register is
// complete when it is used
LBM_D uint32_t tc_ld1(uint32_t taddr) {
    uint32_t r;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r)
        : "r"(taddr)
        : "memory");
    return r;
}

// ---- per CTA ------------------------------------------------------------------------------------------
// every thread of the CTA: warp 0 allocates the TMEM columns (and gives up the right to allocate more,
// so other CTAs on the SM may), thread 0 initialises the mbarrier, the weight image is copied in and
// k group 1 of the layer-1 operand (inputs 8..15) zeroed; returns the TMEM base address
LBM_D uint32_t tc_setup(TcSmem& s, const uint4* img) {
    const int t = threadIdx.x, nt = blockDim.x;
    if (t < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s.tmem)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (t == 0) {
        mbar_init(&s.bar, 1);
        fence_mbar_init();
    }
    for (int i = t; i < kTcWRows; i += nt) s.w[i] = img[i];
    const uint4 z = make_uint4(0, 0, 0, 0);
    for (int r = t; r < 128; r += nt) {
        s.a1[0][tc_off(r, 1, 2) / 16] = z;
        s.a1[1][tc_off(r, 1, 2) / 16] = z;
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    return s.tmem;
}
// every thread of the CTA, after its last tcgen05.ld: warp 0 frees the columns
LBM_D void tc_teardown(uint32_t tm) {
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(kTcCols) : "memory");
    }
}

// one layer's products for both tiles: the CTA synchronises (every thread has stored its rows of the A
// operands and fenced them for the async proxy), thread 0 issues the MMAs and commits them to the
// mbarrier
template <int LAYER>
LBM_D void tc_issue(TcSmem& s, uint32_t tm) {
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
        tc_fence_after();
        const char* w = reinterpret_cast<const char*>(s.w);
#pragma unroll
        for (int tile = 0; tile < 2; tile++) {
            if constexpr (LAYER == 1) {
                tc_mma(tm + (uint32_t)(kTcH * tile), tc_desc(s.a1[tile], 256), tc_desc(w + kTcW1, 256), tc_idesc(kTcH), 0);
            } else {
                constexpr int N = LAYER == 2 ? kTcH : 16;
                const char* wb = w + (LAYER == 2 ? kTcW2 : kTcW3);
                const char* a = reinterpret_cast<const char*>(s.a2[tile]);
#pragma unroll
                for (int kk = 0; kk < kTcH / 16; kk++)  // K = H as K = 16 steps (two k groups each)
                    tc_mma(tm + (uint32_t)(N * tile), tc_desc(a + kk * 256, kTcKG * 128),
                           tc_desc(wb + kk * 256, kTcKG * 128), tc_idesc(N), (uint32_t)kk);
            }
        }
        tc_commit(&s.bar);
    }
}
// wait for the products of `phase`: thread 0 polls the mbarrier (bounded) while the other threads block
// in the CTA barrier, which costs them no issue slots (every thread polling measured 1.2x the warp
// instructions of the kernel).  A CTA that gives up records DEV_ERR_MMA_TIMEOUT and waits once more
// (bounded) so that nothing is in flight when its TMEM is freed.
LBM_D void tc_wait(TcSmem& s, unsigned phase, int* err) {
    if (threadIdx.x == 0 && !mbar_wait_bounded(&s.bar, phase)) {
        if (err) atomicExch(err, DEV_ERR_MMA_TIMEOUT);
        mbar_wait_bounded(&s.bar, phase);
    }
    __syncthreads();
    tc_fence_after();
}

// 16 consecutive 32-bit columns of this thread's lane, complete on return
LBM_D void tc_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}

// a layer's accumulators of this thread's row in one tile (H columns at `col`) -> + bias -> activation ->
// FP16 -> the next operand's row (k groups 0 .. H/8 - 1)
template <bool BIAS>
LBM_D void tc_act_row(uint32_t lane_addr, int col, const float* bias, uint4* a2tile) {
    const int t = threadIdx.x;
#pragma unroll
    for (int half = 0; half < kTcH / 16; half++) {
        uint32_t r[16];
        tc_ld16(lane_addr + (uint32_t)(col + 16 * half), r);
#pragma unroll
        for (int q = 0; q < 2; q++) {
            F2 v[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int c = 8 * q + 2 * i;  // column within the 16 loaded
                v[i] = F2(__uint_as_float(r[c]), __uint_as_float(r[c + 1]));
                if constexpr (BIAS) v[i] = v[i] + F2(bias[16 * half + c], bias[16 * half + c + 1]);  // one packed add per two columns
            }
            uint4 h;
            h.x = mlp_act(v[0].v.x, v[0].v.y);
            h.y = mlp_act(v[1].v.x, v[1].v.y);
            h.z = mlp_act(v[2].v.x, v[2].v.y);
            h.w = mlp_act(v[3].v.x, v[3].v.y);
            a2tile[tc_off(t, 2 * half + q, kTcKG) / 16] = h;
        }
    }
}

// output pre-activation z (without b3) of this thread's two cells; rowA / rowB: their input rows (8
// halves: 7 normalised inputs and 1).  Every thread of the CTA calls it; a call completes three phases of
// the mbarrier, so `parity` (the parity of the first) alternates from call to call on one tc_setup.
LBM_D float2 tc_mlp(TcSmem& s, uint32_t tm, uint4 rowA, uint4 rowB, const MlpNorm& nm, int* err, unsigned parity) {
    const int t = threadIdx.x;
    const uint32_t lane_addr = tm + ((uint32_t)(t & ~31) << 16);  // lane field: first lane of this warp
    s.a1[0][tc_off(t, 0, 2) / 16] = rowA;
    s.a1[1][tc_off(t, 0, 2) / 16] = rowB;
    tc_issue<1>(s, tm);
    tc_wait(s, parity, err);
    tc_act_row<false>(lane_addr, 0, nullptr, s.a2[0]);
    tc_act_row<false>(lane_addr, kTcH, nullptr, s.a2[1]);
    tc_issue<2>(s, tm);
    tc_wait(s, parity ^ 1u, err);
    tc_act_row<true>(lane_addr, 0, nm.b2, s.a2[0]);
    tc_act_row<true>(lane_addr, kTcH, nm.b2, s.a2[1]);
    tc_issue<3>(s, tm);
    tc_wait(s, parity, err);
    const float zA = __uint_as_float(tc_ld1(lane_addr + 0));
    const float zB = __uint_as_float(tc_ld1(lane_addr + 16));
    tc_fence_before();  // a later call's first barrier orders these loads before its products
    return make_float2(zA, zB);
}

}  // namespace lbm
