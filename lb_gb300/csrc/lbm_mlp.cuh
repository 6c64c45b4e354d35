// lbm_mlp.cuh - learned LES closure: strain-rate features, the per-warp tensor-core MLP evaluated
// inside the step kernel, and the activation shared with the training kernels.
//
// Network: x(7) -> H -> H -> 1 (H = kMlpHid = 32), GELU in its sigmoid form g(x) = x sigmoid(1.702 x)
// after both hidden layers, nu_t = out_scale * softplus(z).  Inputs (order of lbm.h) from the strain
// rate S and rho:
//   0 tr S   1 I2 = (tr^2 S - S:S)/2   2 I3 = det S   3 Lode parameter 3 sqrt(6) det(S_d) / |S_d|^3
//   4 S_d:S_d / S:S   5 rho   6 |S| = sqrt(2 S:S)
// normalised as (x - mean) / std.
//
// Step-kernel evaluation (FP16 operands, all in registers of one warp; layer 1, eight products per sum,
// accumulates in FP16, layers 2 and 3 in FP32): the 64
// cells of a warp (two per lane) are staged as 64 rows of 8 halves (7 inputs and a 1 that carries the
// first bias) and loaded as A fragments with ldmatrix; layer 1 is mma.m16n8k8, layers 2 and 3
// mma.m16n8k16.  The accumulator fragment of one layer (rows g, g+8, columns 2c, 2c+1 of each n-tile)
// is the A fragment of the next after packing to f16x2, so no data moves between lanes.  The activation
// is applied as z (1 + tanh z) with z = 0.851 x (g(x) = x/2 (1 + tanh(0.851 x)) exactly), the factors
// 0.851 and 1/1.702 being folded into the FP16 weights on the host: one tanh.approx.f16x2 and one HFMA2
// per two elements.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include "lbm_math.cuh"

namespace lbm {

constexpr int kMlpIn = 7, kMlpHid = 32, kMlpSample = 10;
constexpr float kGeluA = 1.702f;
constexpr int kMlpParams = kMlpHid * kMlpHid + 10 * kMlpHid + 1;
// offsets into the FP32 parameter vector: w1[H][7], b1[H], w2[H][H], b2[H], w3[H], b3
constexpr int kMlpW1 = 0, kMlpB1 = 7 * kMlpHid, kMlpW2 = 8 * kMlpHid, kMlpB2 = kMlpW2 + kMlpHid * kMlpHid,
              kMlpW3 = kMlpB2 + kMlpHid, kMlpB3 = kMlpW3 + kMlpHid;
// warp evaluation: n-tiles of 8 hidden units, k16 steps over the hidden units
constexpr int kMlpNT = kMlpHid / 8, kMlpKS = kMlpHid / 16;
static_assert(kMlpHid == 16 || kMlpHid == 32, "the fragment table holds up to four n-tiles");
// uint4 rows of the fragment table: [0] W1, [1..4] W2 n-tiles, [5] W3, [6..7] b2 (as floats); the
// device buffer holds the table ([kMlpFragRows][32]) followed by the tcgen05 weight image
// (kMlpTcRows uint4, lbm_mlp_tc.cuh)
constexpr int kMlpFragRows = 8;
// tcgen05 image: W1 H x 16, W2 H x H, W3 16 x H halves
constexpr int kMlpTcRows = (kMlpHid * 16 + kMlpHid * kMlpHid + 16 * kMlpHid) * 2 / 16;
constexpr int kMlpFragTotal = kMlpFragRows * 32 + kMlpTcRows;

// ---- features -------------------------------------------------------------------------------------
LBM_D float lmax(float a, float b) { return fmaxf(a, b); }
LBM_D float lmin(float a, float b) { return fminf(a, b); }
LBM_D F2 lmax(F2 a, F2 b) { return F2(fmaxf(a.v.x, b.v.x), fmaxf(a.v.y, b.v.y)); }
LBM_D F2 lmin(F2 a, F2 b) { return F2(fminf(a.v.x, b.v.x), fminf(a.v.y, b.v.y)); }
LBM_D float rsqrt_pos(float x) { return rsqrtf(fmaxf(x, 1e-30f)); }
LBM_D F2 rsqrt_pos(F2 x) { return F2(rsqrt_pos(x.v.x), rsqrt_pos(x.v.y)); }

// s = (xx, yy, zz, xy, xz, yz) of S in lattice units
template <class L>
LBM_D void mlp_features(const L (&s)[6], L rho, L (&x)[7]) {
    const L tr = s[0] + s[1] + s[2];
    const L off2 = lfma(s[3], s[3], lfma(s[4], s[4], s[5] * s[5]));
    const L s2 = lfma(s[0], s[0], lfma(s[1], s[1], lfma(s[2], s[2], off2 + off2)));  // S:S
    // det of a symmetric matrix with diagonal (a, b, c): a (b c - yz^2) - xy (xy c - yz xz) + xz (xy yz - b xz)
    auto det3 = [&](L a, L b, L c) {
        const L m0 = lfma(b, c, -(s[5] * s[5]));
        const L m1 = lfma(s[3], c, -(s[5] * s[4]));
        const L m2 = lfma(s[3], s[5], -(b * s[4]));
        return lfma(a, m0, lfma(-s[3], m1, s[4] * m2));
    };
    const L t3 = tr * (L)(1.0f / 3.0f);
    const L d2 = lfma(-tr, t3, s2);  // S_d:S_d
    const L detd = det3(s[0] - t3, s[1] - t3, s[2] - t3);
    const L id = rsqrt_pos(d2);
    L lode = (L)7.348469228f * detd * (id * id * id);  // 3 sqrt(6)
    lode = lmin(lmax(lode, (L)-1.0f), (L)1.0f);
    x[0] = tr;
    x[1] = (L)0.5f * lfma(tr, tr, -s2);
    x[2] = det3(s[0], s[1], s[2]);
    x[3] = lode;
    x[4] = d2 * rcp(lmax(s2, (L)1e-30f));
    x[5] = rho;
    x[6] = sqrt_pos(s2 + s2);
}

// ---- training-side activations (FP32) -------------------------------------------------------------
LBM_D float sigmoidf_(float x) { return 1.0f / (1.0f + expf(-x)); }
LBM_D float gelu_s(float x) { return x * sigmoidf_(kGeluA * x); }
LBM_D float gelu_s_grad(float x) {
    const float s = sigmoidf_(kGeluA * x);
    return s + kGeluA * x * s * (1.0f - s);
}
LBM_D float softplusf_(float z) { return fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z))); }
// the step kernel's softplus (fast exponential and logarithm)
LBM_D float softplus_fast(float z) { return fmaxf(z, 0.0f) + __logf(1.0f + __expf(-fabsf(z))); }

// ---- warp-level tensor-core evaluation ------------------------------------------------------------
LBM_D uint32_t h2_bits(__half2 h) { return *reinterpret_cast<uint32_t*>(&h); }
LBM_D __half2 bits_h2(uint32_t u) { return *reinterpret_cast<__half2*>(&u); }

// z (1 + tanh z) on a packed pair of accumulators (z already carries the folded 0.851), lo in the lower
// half of the f16x2 result
LBM_D uint32_t mlp_act(float lo, float hi) {
    const __half2 z = __floats2half2_rn(lo, hi);
    uint32_t t;
    asm("tanh.approx.f16x2 %0, %1;" : "=r"(t) : "r"(h2_bits(z)));
    return h2_bits(__hfma2(z, bits_h2(t), z));
}

// z (1 + tanh z) on a packed pair already in FP16
LBM_D uint32_t mlp_act_h(uint32_t zb) {
    uint32_t t;
    asm("tanh.approx.f16x2 %0, %1;" : "=r"(t) : "r"(zb));
    return h2_bits(__hfma2(bits_h2(zb), bits_h2(t), bits_h2(zb)));
}

// layer 1 (K = 8, the bias in the eighth column): FP16 accumulators from zero; the sums go to the
// activation in FP16 either way, so no FP32-to-FP16 pack
LBM_D void mma_k8_h(uint32_t (&d)[2], uint32_t a0, uint32_t a1, uint32_t b0) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f16.f16.f16.f16 {%0,%1}, {%2,%3}, {%4}, {%5,%5};"
        : "=r"(d[0]), "=r"(d[1])
        : "r"(a0), "r"(a1), "r"(b0), "r"(0u));
}

LBM_D void mma_k8(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t b0) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(b0));
}
LBM_D void mma_k16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}
// the same with a separate accumulator input z in every element (zero here): the output registers are
// not also the input, so no copy of a zero or bias quad precedes each product (fewer moves and spills;
// the layer-2 bias is added after the product with one packed add per two elements)
LBM_D void mma_k8_z(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t b0, float z) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%7,%7,%7,%7};"
        : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
        : "r"(a0), "r"(a1), "r"(b0), "f"(z));
}
LBM_D void mma_k16_z(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0, uint32_t b1, float z) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%10,%10,%10,%10};"
        : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1), "f"(z));
}
LBM_D void ldmatrix_x4(uint32_t (&r)[4], const void* smem_row) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(smem_row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

// normalisation and training range of the inputs (uniform over the launch):
// normalised input = fma(x, isd, nmi) with isd = 1/std, nmi = -mean/std (rounded to FP32)
struct MlpNorm {
    float isd[7], nmi[7], lo[7], hi[7];
    float b3, scale;
    float b2[kMlpHid];  // layer-2 bias, 0.851 folded in (the tcgen05 path adds it after the accumulator load)
};

// normalised inputs of one cell as a row of 8 halves (input 7 = 1), and whether all lie in range
LBM_D uint4 mlp_row(const float (&x)[7], const MlpNorm& nm, bool& in_range) {
    float h[8];
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 7; i++) {
        h[i] = fmaf(x[i], nm.isd[i], nm.nmi[i]);
        ok = ok && h[i] >= nm.lo[i] && h[i] <= nm.hi[i];
    }
    h[7] = 1.0f;
    in_range = ok;
    uint4 r;
    r.x = h2_bits(__floats2half2_rn(h[0], h[1]));
    r.y = h2_bits(__floats2half2_rn(h[2], h[3]));
    r.z = h2_bits(__floats2half2_rn(h[4], h[5]));
    r.w = h2_bits(__floats2half2_rn(h[6], h[7]));
    return r;
}
// the same for the two cells of a packed pair (one FFMA2 per input)
LBM_D void mlp_rows2(const F2 (&x)[7], const MlpNorm& nm, uint4& ra, uint4& rb, bool& ia, bool& ib) {
    F2 h[7];
    bool oa = true, ob = true;
#pragma unroll
    for (int i = 0; i < 7; i++) {
        h[i] = lfma(x[i], F2(nm.isd[i]), F2(nm.nmi[i]));
        oa = oa && h[i].v.x >= nm.lo[i] && h[i].v.x <= nm.hi[i];
        ob = ob && h[i].v.y >= nm.lo[i] && h[i].v.y <= nm.hi[i];
    }
    ia = oa;
    ib = ob;
    ra.x = h2_bits(__floats2half2_rn(h[0].v.x, h[1].v.x));
    ra.y = h2_bits(__floats2half2_rn(h[2].v.x, h[3].v.x));
    ra.z = h2_bits(__floats2half2_rn(h[4].v.x, h[5].v.x));
    ra.w = h2_bits(__floats2half2_rn(h[6].v.x, 1.0f));
    rb.x = h2_bits(__floats2half2_rn(h[0].v.y, h[1].v.y));
    rb.y = h2_bits(__floats2half2_rn(h[2].v.y, h[3].v.y));
    rb.z = h2_bits(__floats2half2_rn(h[4].v.y, h[5].v.y));
    rb.w = h2_bits(__floats2half2_rn(h[6].v.y, 1.0f));
}

// Output pre-activation z (without b3) of the two cells of every lane.  Rows: lane l's first cell is
// row l, its second row 32 + l.  stage: this warp's 64 x 16 B of shared memory; wf: the fragment table
// [kMlpFragRows][32] in shared memory.  Every lane of the warp must call it.
// 128-bit shared-memory load that the compiler keeps where it is written (re-read per m-tile instead
// of holding the 16 W2 registers across the whole evaluation)
LBM_D uint4 lds128(const uint4* p) {
    uint4 r;
    asm volatile("ld.shared.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
                 : "r"((unsigned)__cvta_generic_to_shared(p)));
    return r;
}

LBM_D float2 mlp_warp(uint4 rowA, uint4 rowB, uint4* stage, const uint4 (*wf)[32]) {
    const int lane = threadIdx.x & 31;
    stage[lane] = rowA;
    stage[32 + lane] = rowB;
    __syncwarp();
    uint32_t a[8];
    {
        uint32_t r[4];
        ldmatrix_x4(r, stage + lane);       // m-tiles 0, 1 (rows 0..31)
        a[0] = r[0]; a[1] = r[1]; a[2] = r[2]; a[3] = r[3];
        ldmatrix_x4(r, stage + 32 + lane);  // m-tiles 2, 3 (rows 32..63)
        a[4] = r[0]; a[5] = r[1]; a[6] = r[2]; a[7] = r[3];
    }
    __syncwarp();                            // the stage takes the outputs below
    float* out = reinterpret_cast<float*>(stage);
    const uint4 w1 = lds128(&wf[0][lane]);
    const uint4 w3 = lds128(&wf[5][lane]);
    const uint4 bA = lds128(&wf[6][lane]), bB = lds128(&wf[7][lane]);
    const uint32_t w1j[4] = {w1.x, w1.y, w1.z, w1.w};
    const uint32_t w3k[4] = {w3.x, w3.y, w3.z, w3.w};
    const uint32_t b2[4][2] = {{bA.x, bA.y}, {bA.z, bA.w}, {bB.x, bB.y}, {bB.z, bB.w}};
#pragma unroll
    for (int t = 0; t < 4; t++) {
        uint32_t h[kMlpNT][2];
#pragma unroll
        for (int j = 0; j < kMlpNT; j++) {
            uint32_t d[2];
            mma_k8_h(d, a[2 * t], a[2 * t + 1], w1j[j]);
            h[j][0] = mlp_act_h(d[0]);
            h[j][1] = mlp_act_h(d[1]);
        }
        uint32_t h2[kMlpNT][2];
#pragma unroll
        for (int j = 0; j < kMlpNT; j++) {
            const uint4 w2 = lds128(&wf[1 + j][lane]);
            const uint32_t w2k[4] = {w2.x, w2.y, w2.z, w2.w};
            const float c0 = __uint_as_float(b2[j][0]), c1 = __uint_as_float(b2[j][1]);
            float d[4];
            mma_k16_z(d, h[0][0], h[0][1], h[1][0], h[1][1], w2k[0], w2k[1], 0.0f);
#pragma unroll
            for (int ks = 1; ks < kMlpKS; ks++)
                mma_k16(d, h[2 * ks][0], h[2 * ks][1], h[2 * ks + 1][0], h[2 * ks + 1][1], w2k[2 * ks], w2k[2 * ks + 1]);
            const F2 e0 = F2(d[0], d[1]) + F2(c0, c1), e1 = F2(d[2], d[3]) + F2(c0, c1);
            h2[j][0] = mlp_act(e0.v.x, e0.v.y);
            h2[j][1] = mlp_act(e1.v.x, e1.v.y);
        }
        float d[4];
        mma_k16_z(d, h2[0][0], h2[0][1], h2[1][0], h2[1][1], w3k[0], w3k[1], 0.0f);
#pragma unroll
        for (int ks = 1; ks < kMlpKS; ks++)
            mma_k16(d, h2[2 * ks][0], h2[2 * ks][1], h2[2 * ks + 1][0], h2[2 * ks + 1][1], w3k[2 * ks], w3k[2 * ks + 1]);
        if ((lane & 3) == 0) {  // column 0: rows g and g+8 of m-tile t
            out[16 * t + (lane >> 2)] = d[0];
            out[16 * t + 8 + (lane >> 2)] = d[2];
        }
    }
    __syncwarp();
    const float2 z = make_float2(out[lane], out[32 + lane]);
    __syncwarp();
    return z;
}

// eddy viscosity from the output pre-activation
LBM_D float mlp_nu(float z, const MlpNorm& nm) { return nm.scale * softplus_fast(z + nm.b3); }

}  // namespace lbm
