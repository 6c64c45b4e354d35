// lbm_step_mlp.cuh - the pair step kernel with the learned closure (LBM_CLOSURE_MLP, FP32 and
// FP16-deviation storage).
//
// Same loads, collision and stores as k_step2; only the relaxation rate differs.  Per packed pair:
//   1. moments and the non-equilibrium stress Pi = M - rho (u u + I/3), as the Smagorinsky closure;
//   2. the Smagorinsky relaxation time tau_S (OmegaLES.h:117-124) and from it the strain-rate estimate
//      S = -3 Pi / (2 rho tau_S), which is exact when the cell relaxed with tau_S (Pi = -2/3 rho tau S);
//   3. the seven inputs of S and rho, normalised, as FP16 rows; the warp's 64 cells go through the
//      tensor-core MLP together (mlp_warp, warp-level mma.sync), so every lane reaches it, including
//      lanes without a pair; with LBM_OPT_MLP_TCGEN05 the plain rows' CTA of 256 cells goes through
//      tcgen05.mma with TMEM accumulators instead (tc_mlp, lbm_mlp_tc.cuh);
//   4. tau = tau_0 + 3 nu_t for cells whose inputs lie in the training range, tau_S otherwise.
// Cells that are not packed bulk pairs take the per-cell path with the Smagorinsky closure; the rows beside
// a flat wall (every cell such a cell) run the packed wall kernel with the Smagorinsky closure instead.
// MODE 0: the network runs in this step.  MODE 1: it runs and its nu_t (or -1 for the fallback) is kept
// per cell in FP16 (Params::nut).  MODE 2: it does not run; each pair relaxes with the kept nu_t (the
// Smagorinsky rate where the kept value is negative or not a number), fetched before the populations.
// The plain rows' MODE 2 steps run k_step2_plain with closure 2 (step_pair_plain, the same rate), the
// register allocation of the Smagorinsky plain-row kernel.
#pragma once

#include "lbm_mlp.cuh"
#include "lbm_mlp_tc.cuh"
#include "lbm_step.cuh"

namespace lbm {

// resident CTAs per SM requested from the register allocator: none for the steps that run the network
// (6 and 7 measured no faster), as k_step2 (step2_min_blocks) for the steps that reuse kept nu_t
#ifndef LBM_MLP_MIN_BLOCKS
#define LBM_MLP_MIN_BLOCKS 0
#endif
// the plain-row kernel that runs the network: 7 CTAs per SM (72 registers) measured 27.9 GLUPS against
// 27.6 at 6 (80 registers) with the 7-32-32-1 GELU network
#ifndef LBM_MLP_PLAIN_MIN_BLOCKS
#define LBM_MLP_PLAIN_MIN_BLOCKS 7
#endif
// ROWS: 0 one launch over the lattice (grid x = pair block, y, z); 1 the plain rows of the split step
// (every pair a packed bulk pair off the y/z seams, lbm_step.cuh); 2 the remaining rows (1-D grid of
// listed rows x pair blocks, row_block)
constexpr int mlp_min_blocks(int mode, int rows, int coll) {
    return mode == 2 ? step2_min_blocks(coll) : (rows == 1 ? LBM_MLP_PLAIN_MIN_BLOCKS : LBM_MLP_MIN_BLOCKS);
}
// one x-pair of the learned-closure step (x0 even; y, z for ROWS 0 and 2, row r for ROWS 1).  Every
// thread of the warp (TC: of the CTA) calls it, including threads without a pair, since the network runs
// for the warp's (CTA's) cells together.
template <class S, int COLL, bool ODD, int MODE, int ROWS, bool TC, class TS>
LBM_D void mlp_pair(const Params& p, int x0, int y, int z, int r, const uint4 (*wf)[32], uint4* stage, TS& ts,
                    uint32_t tm, unsigned parity) {
    unsigned idx0;
    const bool live = x0 < p.nx;
    const bool two = x0 + 1 < p.nx;
    if constexpr (ROWS == 1) idx0 = (unsigned)(live ? x0 : 0) + (unsigned)p.nx * (unsigned)r;
    else idx0 = (unsigned)(live ? x0 : 0) + (unsigned)p.nx * ((unsigned)y + (unsigned)p.ny * (unsigned)z);
    bool pair;
    if constexpr (ROWS == 1) {
        pair = live;  // plain rows: nx even, every pair packed
    } else {
        const uint8_t f0 = live ? (p.cls[idx0] & (uint8_t)~BIT_REFBULK) : (uint8_t)0;
        const uint8_t f1 = two ? (p.cls[idx0 + 1] & (uint8_t)~BIT_REFBULK) : (uint8_t)0;
        pair = two && f0 == CLS_BULK && f1 == CLS_BULK && (p.nx & 1) == 0;
    }

    const PairCodec k = make_codec<S>(p);
    const bool yz_seam = ROWS != 1 &&
        ((p.wrap[1] && (y == 0 || y == p.ny - 1)) || (p.wrap[2] && (z == 0 || z == p.nz - 1)));
    const PairIdx q = make_pair_idx(p, (int)idx0, x0);

    float2 kept = make_float2(-1.f, -1.f);
    if (MODE == 2 && pair) kept = __half22float2(__ldg((const __half2*)(p.nut + idx0)));
    F2 f[27];
    Mom<F2> mm;
    F2 ri, ux, uy, uz, om_s;
    uint4 rowA = make_uint4(0, 0, 0, 0), rowB = rowA;
    bool inA = false, inB = false;
    // FP16 storage + cumulant-2015: the moments come from the raw deviations as in step_pair, so the
    // Smagorinsky fallback rate and the collision see the same roundings as k_step2 (an all-fallback
    // model then reproduces k_step2 bit for bit)
    constexpr bool RAW = S::kind == 2 && COLL == 1;
    if (pair) {
        if (!yz_seam) {
            load_pair<S, ODD, RAW>(p, q, k, f);
        } else {
            PairRows w;
            make_pair_rows(p, x0, y, z, w);
            load_pair_rows<S, ODD, RAW>(p, w, k, f);
        }
        mm = raw_moments(f);
        if constexpr (RAW) mm = moments_from_raw(mm, p);
        ri = rcp(mm.rho);
        ux = mm.jx * ri; uy = mm.jy * ri; uz = mm.jz * ri;
        if (p.has_force) {
            ux = lfma(F2(p.Ff[0]), F2(0.5f), mm.jx) * ri;
            uy = lfma(F2(p.Ff[1]), F2(0.5f), mm.jy) * ri;
            uz = lfma(F2(p.Ff[2]), F2(0.5f), mm.jz) * ri;
        }
        if (p.acc) {
            acc_add(p, idx0, mm.rho.v.x, ux.v.x, uy.v.x, uz.v.x);
            acc_add(p, idx0 + 1, mm.rho.v.y, ux.v.y, uy.v.y, uz.v.y);
        }
        // Pi and tau_S exactly as omega_smagorinsky
        const F2 third = mm.rho * F2(1.0f / 3.0f);
        const F2 rux = mm.rho * ux, ruy = mm.rho * uy, ruz = mm.rho * uz;
        const F2 pxx = lfma(-rux, ux, mm.Mxx - third), pyy = lfma(-ruy, uy, mm.Myy - third),
                 pzz = lfma(-ruz, uz, mm.Mzz - third);
        const F2 pxy = lfma(-rux, uy, mm.Mxy), pxz = lfma(-rux, uz, mm.Mxz), pyz = lfma(-ruy, uz, mm.Myz);
        const F2 off = lfma(pxy, pxy, lfma(pxz, pxz, pyz * pyz));
        const F2 PI2 = lfma(pxx, pxx, lfma(pyy, pyy, lfma(pzz, pzz, off + off)));
        const F2 PI = sqrt_pos(PI2);
        const F2 tau = F2(p.tauf);
        const F2 tles = lfma(tau, F2(0.5f), F2(0.5f) * sqrt_pos(lfma(tau, tau, F2(p.cles18f) * ri * PI)));
        om_s = rcp(tles);
        if constexpr (MODE != 2) {
            // strain rate S = -3 Pi / (2 rho tau_S)
            const F2 sc = F2(-1.5f) * ri * om_s;
            const F2 s[6] = {pxx * sc, pyy * sc, pzz * sc, pxy * sc, pxz * sc, pyz * sc};
            F2 xf[7];
            mlp_features(s, mm.rho, xf);
            mlp_rows2(xf, p.mlp, rowA, rowB, inA, inB);
        }
    }
    float nuA = kept.x, nuB = kept.y;
    if constexpr (MODE != 2) {
        float2 zo;
        if constexpr (TC) zo = tc_mlp(ts, tm, rowA, rowB, p.mlp, p.err, parity);
        else zo = mlp_warp(rowA, rowB, stage, wf);
        nuA = inA ? mlp_nu(zo.x, p.mlp) : -1.0f;
        nuB = inB ? mlp_nu(zo.y, p.mlp) : -1.0f;
        if (MODE == 1 && pair) *(__half2*)(p.nut + idx0) = __floats2half2_rn(nuA, nuB);
    }
    (void)rowA; (void)rowB; (void)inA; (void)inB;
    if (pair) {
        // nu >= 0 is false for the fallback mark (-1) and for a kept value that is not a number
        const F2 om(rate_kept(nuA, p.tauf, om_s.v.x), rate_kept(nuB, p.tauf, om_s.v.y));
        collide_with_rate<COLL>(f, mm, ri, ux, uy, uz, om, p.has_force != 0, F2(p.Ff[0]), F2(p.Ff[1]),
                                F2(p.Ff[2]));
        if (!yz_seam) {
            store_pair<S, ODD>(p, q, k, f);
        } else {
            PairRows w;
            make_pair_rows(p, x0, y, z, w);
            store_pair_rows<S, ODD>(p, w, k, f);
        }
    } else if constexpr (ROWS != 1) {
        if (live) {
            step_cell_call<S, COLL, 1, ODD>(p, x0, y, z);
            if (two) step_cell_call<S, COLL, 1, ODD>(p, x0 + 1, y, z);
        }
    }
}

// TC (plain rows, network steps): the network on tcgen05.mma with TMEM accumulators for the CTA's cells
// (lbm_mlp_tc.cuh) instead of the per-warp mma.sync evaluation
template <class S, int COLL, bool ODD, int MODE, int ROWS = 0, bool TC = false>
__global__ void __launch_bounds__(128, mlp_min_blocks(MODE, ROWS, COLL)) k_step2_mlp(Params p, const int32_t* rows, int nrows) {
    static_assert(S::kind != 0, "the learned closure runs on the packed FP32 path");
    static_assert(!TC || (ROWS == 1 && MODE != 2), "the tcgen05 network serves the plain rows' network steps");
    static_assert(MODE != 2 || ROWS != 1, "the plain rows' steps without the network run k_step2_plain");
    constexpr bool WARP = MODE != 2 && !TC;
    __shared__ uint4 wf[WARP ? kMlpFragRows : 1][32];
    __shared__ uint4 stage[WARP ? 4 : 1][64];
    __shared__ typename std::conditional<TC, TcSmem, char>::type ts;
    if constexpr (WARP) {
        for (int i = threadIdx.x; i < kMlpFragRows * 32; i += blockDim.x) (&wf[0][0])[i] = p.mlp_frag[i];
        __syncthreads();
    }
    int x0, y = 0, z = 0, r = 0;
    if constexpr (ROWS == 0) {
        x0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
        y = blockIdx.y;
        z = blockIdx.z;
    } else {
        if (!row_block(rows, nrows, r, x0)) return;  // tail block past the list: the whole block leaves
        if constexpr (ROWS == 2) {
            y = r % p.ny;
            z = r / p.ny;
        }
    }
    uint32_t tm = 0;
    if constexpr (TC) tm = tc_setup(ts, p.mlp_frag + kMlpFragRows * 32);
    mlp_pair<S, COLL, ODD, MODE, ROWS, TC>(p, x0, y, z, r, wf, stage[WARP ? threadIdx.x >> 5 : 0], ts, tm, 0u);
    if constexpr (TC) tc_teardown(tm);
}

}  // namespace lbm
