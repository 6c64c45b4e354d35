// lbm_step.cuh - the fused collide-and-stream step kernels.
//
// k_step  : one thread per cell (FP64 storage).
// k_step2 : one thread per x-pair of cells (FP32 and FP16-deviation storage).  When both cells are
//           plain bulk cells off the periodic seams, the pair is loaded with 64-bit (FP32) or 32-bit
//           (FP16) accesses where the AA slot pair is aligned and collided in packed FP32 (F2 lanes:
//           FADD2/FMUL2/FFMA2); otherwise each cell takes the scalar per-cell path.
// k_step2_plain / k_step2_list : the same step split by rows (the default): the rows whose pairs all
//           take the packed path, and the remaining rows.
#pragma once

#include "lbm_device.cuh"
#include "lbm_sync.cuh"

namespace lbm {

template <class R> LBM_D R p_om0(const Params& p) { if constexpr (std::is_same<R, float>::value) return p.omega0f; else return p.omega0; }

LBM_D void acc_add(const Params& p, long long i, double rho, double ux, double uy, double uz) {
    double* a = p.acc;
    const long long N = p.N;
    a[i] += rho; a[N + i] += ux; a[2 * N + i] += uy; a[3 * N + i] += uz;
    a[4 * N + i] += ux * ux; a[5 * N + i] += uy * uy; a[6 * N + i] += uz * uz;
    a[7 * N + i] += ux * uy; a[8 * N + i] += ux * uz; a[9 * N + i] += uy * uz;
}

// relaxation rate and collision of one lane (a cell, or a pair of cells); SP: the rate is lowered by
// dom afterwards (the outlet sponge, OutletNeighbourEquilibriumOmega.h:69-74 after TURBULENCETYPE::omega)
template <int COLL, int CLOS, bool SP = false, class L>
LBM_D void collide_lane(L (&f)[27], const Mom<L>& mm, L ri, L ux, L uy, L uz, L tau, L cles18, L om0,
                        bool force, L Fx, L Fy, L Fz, L dom = L(0.0f)) {
    L om;
    if constexpr (CLOS == 0) om = om0;
    else om = omega_smagorinsky(tau, cles18, mm.rho, ri, ux, uy, uz, mm);
    if constexpr (SP) om = om - dom;
    if constexpr (COLL == 0) {
        collide_srt(f, mm.rho, ux, uy, uz, om);
        if (force) srt_force(f, ux, uy, uz, om, Fx, Fy, Fz);
    } else if constexpr (COLL == 2) {
        collide_cum17(f, mm.rho, ri, ux, uy, uz, om);
    } else {
        collide_cum15(f, mm.rho, ri, ux, uy, uz, om, mm);
    }
}

// the outlet sponge's reduction of the relaxation rate at (x, y, z): slope * (coordinate - begin),
// as OutletNeighbourEquilibriumOmega.h:66-71 forms it (real type times the integer distance)
template <class R>
LBM_D R sponge_rate(const Params& p, int x, int y, int z) {
    const int pos = (p.sponge_axis == 0 ? x : p.sponge_axis == 1 ? y : z) - p.sponge_begin;
    if constexpr (std::is_same<R, float>::value) return p.sponge_slopef * (float)pos;
    else return p.sponge_slope * (double)pos;
}

// ---- one cell (scalar lane) --------------------------------------------------------------------------
template <class S, int COLL, int CLOS, bool ODD>
LBM_D void step_cell(const Params& p, int x, int y, int z) {
    using R = typename S::R;
    const unsigned idx = (unsigned)x + (unsigned)p.nx * ((unsigned)y + (unsigned)p.ny * (unsigned)z);
    const uint8_t fl = p.cls[idx];
    const int cl = fl & CLS_MASK;
    if (cl == CLS_SOLID) return;
    R f[27];
    if (cl == CLS_INLET) {
        // node is not updated; only the time average (MomentTimeAvg runs over every cell) needs it
        if (p.acc) {
            Cell c;
            make_cell(p, x, y, z, c);
            inlet_state<S>(p, c, f);
            R rho, jx, jy, jz, ux, uy, uz;
            moments(f, p, rho, jx, jy, jz, ux, uy, uz);
            acc_add(p, idx, rho, ux, uy, uz);
        }
        return;
    }
    const bool fast = cl == CLS_BULK && !on_seam(p, x, y, z);
    if (fast) {
        load_fast<S, ODD>(p, idx, f);
    } else {
        Cell c;
        make_cell(p, x, y, z, c);
        R drag[3] = {0, 0, 0};
        gather<S, ODD, false>(p, c, cl, f, drag);
    }
    const Mom<R> mm = raw_moments(f);
    const R rho = mm.rho, ri = rcp(rho);
    const R ux = (mm.jx + (R)0.5 * p_F<R>(p, 0)) * ri;
    const R uy = (mm.jy + (R)0.5 * p_F<R>(p, 1)) * ri;
    const R uz = (mm.jz + (R)0.5 * p_F<R>(p, 2)) * ri;
    if (fl & (BIT_PROBE1 | BIT_PROBE2)) {
        R* pr = (R*)p.in_probe + (long long)lvl3(p.m) * 3 * p.n_in;
        const int id = p.aux[idx];
        if (fl & BIT_PROBE1) { pr[id] = rho; pr[p.n_in + id] = ux; }
        else pr[2 * p.n_in + id] = ux;
    }
    if (p.acc) acc_add(p, idx, rho, ux, uy, uz);
    // outlet sponge: omega -= slope * (coordinate - first sponge plane), in the storage's real type
    const R dom = (fl & BIT_SPONGE) ? sponge_rate<R>(p, x, y, z) : (R)0;
    if constexpr (COLL == 3) {
        // CollisionCumD3Q27TurbulentCombined.h:1066-1078: reference flag 1 -> 2015, other flags -> 2017
        if (fl & BIT_REFBULK)
            collide_lane<1, CLOS, true>(f, mm, ri, ux, uy, uz, p_tau<R>(p), p_cles18<R>(p), p_om0<R>(p), false, (R)0,
                                        (R)0, (R)0, dom);
        else
            collide_lane<2, CLOS, true>(f, mm, ri, ux, uy, uz, p_tau<R>(p), p_cles18<R>(p), p_om0<R>(p), false, (R)0,
                                        (R)0, (R)0, dom);
    } else {
        collide_lane<COLL, CLOS, true>(f, mm, ri, ux, uy, uz, p_tau<R>(p), p_cles18<R>(p), p_om0<R>(p),
                                       p.has_force != 0, p_F<R>(p, 0), p_F<R>(p, 1), p_F<R>(p, 2), dom);
    }
    // upstream roles exist for the density-interpolated outlet (f* of the cell) and the neighbour-
    // equilibrium outlets (moments); the density-equilibrium outlet has none
    if ((fl & BIT_OUTUP) && p.outlet_kind != OUT_INTERPOLATED && p.outlet_kind != OUT_DENSITY_EQ) {
        // neighbour-equilibrium outlets: the moments this step's collision used (the reference's
        // u_view / rho_view when the outlet pass of this step runs)
        const int e = p.aux[idx];
        R* ms = (R*)p.out_msave + (long long)(p.m & 1) * 4 * p.n_ms;
        ms[e] = rho; ms[p.n_ms + e] = ux; ms[2 * p.n_ms + e] = uy; ms[3 * p.n_ms + e] = uz;
    } else if ((fl & BIT_OUTUP) && p.outlet_kind == OUT_INTERPOLATED) {
        const int id = p.aux[idx];
        const int s = p.out_dir[id];
        R* sv = (R*)p.out_save + (long long)(p.m & 1) * 18 * p.n_out;
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            if constexpr (cx(V) != 0) if (cx(V) == -s) sv[outlet_slot(V) * p.n_out + id] = f[V];
        });
    }
    if (fast) {
        store_fast<S, ODD>(p, idx, f);
        return;
    }
    if (cl == CLS_LID) {
        // InletVelocityMovingWall.h:40-53: for n.c_v > 0, df(x, opp v) = f*_v - 6 w_v rho (c_v . u_w);
        // the other components keep their value.  Written to the next level.
        const int id = p.aux[idx];
        const int nl = p.n_lid;
        const R* cur = (const R*)p.lid_state + (long long)lvl3(p.m) * 27 * nl;
        R* nxt = (R*)p.lid_state + (long long)lvl3(p.m + 1) * 27 * nl;
        const R n0 = p.lid_n[id], n1 = p.lid_n[nl + id], n2 = p.lid_n[2 * nl + id];
        const R w0 = p.lid_u[id], w1 = p.lid_u[nl + id], w2 = p.lid_u[2 * nl + id];
        const R u2 = ux * ux + uy * uy + uz * uz, w2s = w0 * w0 + w1 * w1 + w2 * w2;
        const bool zh = p.inlet_zouhe != 0;
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            constexpr int O = opp(V);
            // component O is set from f*_V when n.c_V > 0, else it keeps its value
            if (n0 * (R)cx(V) + n1 * (R)cy(V) + n2 * (R)cz(V) > (R)0) {
                if (zh)  // InletVelocityZouHe.h:85-97: f*_V - f_eq_V(rho, u) + f_eq_O(rho, u_b)
                    nxt[O * nl + id] = f[V] - feq<V>(rho, ux, uy, uz, u2) + feq<O>(rho, w0, w1, w2, w2s);
                else
                    nxt[O * nl + id] = f[V] - (R)6 * (R)wgt(V) * rho * ((R)cx(V) * w0 + (R)cy(V) * w1 + (R)cz(V) * w2);
            } else {
                nxt[O * nl + id] = cur[O * nl + id];
            }
        });
        return;
    }
    if (cl == CLS_OUTLET && p.outlet_kind != OUT_INTERPOLATED) {
        // the node's part of the next state's entering links (gathered in the next step):
        //   density-equilibrium  f_eq_v(u, rho_b)            (OutletDensityEquilibrium.h:63-67)
        //   neighbour-equilibrium f_eq_v(u, rho_b) - f*_v     (OutletNeighbourEquilibrium.h:104-110: the
        //                         neighbour x + c_v holds f*_v after streaming; its f_eq_v is added in
        //                         the gather)
        // OmegaRF: rho_b (1 - u_x^2 / 2) where u_x < 0 (OutletNeighbourEquilibriumOmegaRF.h:151-155)
        const int id = p.aux[idx];
        const int s = p.out_dir[id];
        R* sv = (R*)p.out_save + (long long)(p.m & 1) * 18 * p.n_out;
        R rb = (R)p.out_rho[id];
        if (p.outlet_kind == OUT_NEQ_OMEGA_RF && ux < (R)0) rb = (R)((double)rb - 0.5 * (double)ux * (double)ux * (double)rb);
        const R u2 = ux * ux + uy * uy + uz * uz;
        const bool neq = p.outlet_kind != OUT_DENSITY_EQ;
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            if constexpr (cx(V) != 0)
                if (cx(V) == -s) sv[(9 + outlet_slot(V)) * p.n_out + id] = feq<V>(rb, ux, uy, uz, u2) - (neq ? f[V] : (R)0);
        });
    } else if (cl == CLS_OUTLET) {
        const int id = p.aux[idx];
        const int s = p.out_dir[id];
        R* sv = (R*)p.out_save + (long long)(p.m & 1) * 18 * p.n_out;
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            if constexpr (cx(V) != 0) if (cx(V) == -s) sv[(9 + outlet_slot(V)) * p.n_out + id] = f[V];
        });
    }
    Cell c;
    make_cell(p, x, y, z, c);
    scatter<S, ODD>(p, c, f);
}

// out-of-line copy for the pair kernel's fallback, so the packed hot path stays compact in the
// instruction cache
template <class S, int COLL, int CLOS, bool ODD>
__device__ __noinline__ void step_cell_call(const Params& p, int x, int y, int z) {
    step_cell<S, COLL, CLOS, ODD>(p, x, y, z);
}

// COLL: 0 SRT, 1 cumulant-2015, 2 cumulant-2017, 3 combined (2015 on reference flag 1, else 2017).
// CLOS: 0 none, 1 Smagorinsky.
template <class S, int COLL, int CLOS, bool ODD>
__global__ void __launch_bounds__(128) k_step(Params p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= p.nx) return;
    step_cell<S, COLL, CLOS, ODD>(p, x, blockIdx.y, blockIdx.z);
}

template <int COLL, class L>
LBM_D void collide_with_rate(L (&f)[27], const Mom<L>& mm, L ri, L ux, L uy, L uz, L om, bool force, L Fx, L Fy,
                             L Fz) {
    if constexpr (COLL == 0) {
        collide_srt(f, mm.rho, ux, uy, uz, om);
        if (force) srt_force(f, ux, uy, uz, om, Fx, Fy, Fz);
    } else {
        collide_cum15(f, mm.rho, ri, ux, uy, uz, om, mm);
    }
}

// relaxation rate of a cell with a kept learned eddy viscosity: 1/(tau + 3 nu_t), or the Smagorinsky
// rate where the kept value is negative (fallback mark) or not a number
LBM_D float rate_kept(float nu, float tau, float om_s) { return nu >= 0.0f ? __fdividef(1.0f, lfma(3.0f, nu, tau)) : om_s; }

// moments of the populations from those of the stored FP16 deviations, f_v = h_v 2^-s + w_v rho0:
// rho = 2^-s sum h + sum w rho0, j = 2^-s j_h, M_ab = 2^-s M_ab,h + delta_ab sum w rho0 c_x^2 (the
// weights are symmetric, so the odd and mixed sums of w_v rho0 vanish)
LBM_D Mom<F2> moments_from_raw(const Mom<F2>& m, const Params& p) {
    const F2 s = F2(p.inv_scale), d = F2(p.raw_mdiag);
    Mom<F2> o;
    o.rho = lfma(m.rho, s, F2(p.raw_rho));
    o.jx = m.jx * s; o.jy = m.jy * s; o.jz = m.jz * s;
    o.Mxx = lfma(m.Mxx, s, d); o.Myy = lfma(m.Myy, s, d); o.Mzz = lfma(m.Mzz, s, d);
    o.Mxy = m.Mxy * s; o.Mxz = m.Mxz * s; o.Myz = m.Myz * s;
    return o;
}

// moments, relaxation rate and collision of a packed pair of bulk cells
// (time-average accumulation of the two cells idx0, idx0+1 when p.acc is set).  RAW: f holds the FP16
// deviations (the cumulant-2015 collision rebuilds every population from the moments).  CLOS 2 (the
// learned closure in a step that reuses its kept nu_t): each cell relaxes with rate_kept of its kept
// value, the Smagorinsky rate where that is the fallback mark
template <int COLL, int CLOS, bool RAW = false>
LBM_D void collide_pair(const Params& p, F2 (&f)[27], long long idx0, float2 kept = make_float2(-1.f, -1.f)) {
    static_assert(!RAW || COLL == 1, "only the cumulant-2015 step needs no decoded populations");
    Mom<F2> mm = raw_moments(f);
    if constexpr (RAW) mm = moments_from_raw(mm, p);
    const F2 ri = rcp(mm.rho);
    F2 ux = mm.jx * ri, uy = mm.jy * ri, uz = mm.jz * ri;
    if (p.has_force) {
        ux = lfma(F2(p.Ff[0]), F2(0.5f), mm.jx) * ri;
        uy = lfma(F2(p.Ff[1]), F2(0.5f), mm.jy) * ri;
        uz = lfma(F2(p.Ff[2]), F2(0.5f), mm.jz) * ri;
    }
    if (p.acc) {
        acc_add(p, idx0, mm.rho.v.x, ux.v.x, uy.v.x, uz.v.x);
        acc_add(p, idx0 + 1, mm.rho.v.y, ux.v.y, uy.v.y, uz.v.y);
    }
    if constexpr (CLOS == 2) {
        const F2 om_s = omega_smagorinsky(F2(p.tauf), F2(p.cles18f), mm.rho, ri, ux, uy, uz, mm);
        const F2 om(rate_kept(kept.x, p.tauf, om_s.v.x), rate_kept(kept.y, p.tauf, om_s.v.y));
        collide_with_rate<COLL>(f, mm, ri, ux, uy, uz, om, p.has_force != 0, F2(p.Ff[0]), F2(p.Ff[1]),
                                F2(p.Ff[2]));
    } else {
        collide_lane<COLL, CLOS>(f, mm, ri, ux, uy, uz, F2(p.tauf), F2(p.cles18f), F2(p.omega0f),
                                 p.has_force != 0, F2(p.Ff[0]), F2(p.Ff[1]), F2(p.Ff[2]));
    }
}

// ---- x-pairs in packed FP32 ----------------------------------------------------------------------------
// Cells idx0 (even x0) and idx0+1 of a bulk pair.  Even steps touch only the pair's own slots and odd
// steps with c_x = 0 a pair in a neighbouring row: one aligned 64-bit (FP32) / 32-bit (FP16) access.
// Odd steps with c_x != 0 touch an x-shifted pair that straddles the alignment, fetched as two
// scalars.  Relative to the per-direction pointers (which already carry the neighbour offset):
//   read  c_x = +1: cells (x0-1, x0)   -> elements (eL, e1);  c_x = -1: (x0+1, x0+2) -> (e0, eR)
//   write c_x = +1: cells (x0+1, x0+2) -> elements (e0, eR);  c_x = -1: (x0-1, x0)   -> (eL, e1)
// with e0 = idx0, e1 = idx0+1, and eL / eR the same shifted by +-nx where x0-1 / x0+2 wraps across
// a periodic x seam.
struct PairIdx {
    int e0, e1, eL, eR;  // signed: a wrapped index may sit below e0 by up to nx
};
// FP16 codec constants of the four weight classes (w rho0, -w rho0 2^s) as packed pairs
struct PairCodec {
    F2 inv_scale, scale, wr[4], nwrs[4];
};

// element i of a slot array of FP16 values as the slot's base address plus a zero-extended 32-bit
// byte offset (i < 2^31, so 2 i fits): a 64-bit addition on the integer ALU instead of a wide integer
// multiply-add on the FMA pipe, which bounds the FP16 step (measured 45.7 -> 47.3 GLUPS at 512x256x256)
template <class T>
LBM_D T* at32(T* base, int i) {
    static_assert(sizeof(T) == 2, "32-bit byte offsets cover 2^31 elements of 2 bytes");
    return (T*)((char*)base + (uint32_t)i * 2u);
}
template <class T>
LBM_D const T* at32(const T* base, int i) {
    static_assert(sizeof(T) == 2, "32-bit byte offsets cover 2^31 elements of 2 bytes");
    return (const T*)((const char*)base + (uint32_t)i * 2u);
}

// direction V of a pair through the address table of an odd (TODD) or even step: the odd table reads the
// x-shifted pair of cell x - c_V's opposite slot, the even one the pair's own slot V.  RAW (FP16
// storage): the stored deviation h_v itself (the caller then takes the moments of f from those of h,
// moments_from_raw); else the population h_v 2^-s + w_v rho0
template <class S, bool TODD, bool RAW, int V>
LBM_D F2 load_dir(const Params& p, const PairIdx& q, const PairCodec& k) {
    using T = typename S::T;
    constexpr bool split = TODD && cx(V) != 0;
    const int i0 = cx(V) > 0 ? q.eL : q.e0, i1 = cx(V) > 0 ? q.e1 : q.eR;
    if constexpr (S::kind == 1) {
        const T* a = (const T*)(TODD ? p.rd_odd[V] : p.rd_even[V]);
        if constexpr (split) return F2(__ldg(a + i0), __ldg(a + i1));
        else return F2(__ldg((const float2*)(a + q.e0)));
    } else {
        const T* b = (const T*)(TODD ? p.rd_odd[V] : p.rd_even[V]);
        float2 t;
        if constexpr (split) t = make_float2(__half2float(__ldg(at32(b, i0))), __half2float(__ldg(at32(b, i1))));
        else t = __half22float2(__ldg((const __half2*)at32(b, q.e0)));
        if constexpr (RAW) return F2(t);
        else return lfma(F2(t), k.inv_scale, k.wr[csq(V)]);
    }
}
template <class S, bool ODD, bool RAW = false>
LBM_D void load_pair(const Params& p, const PairIdx& q, const PairCodec& k, F2 (&f)[27]) {
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        f[V] = load_dir<S, ODD, RAW, V>(p, q, k);
    });
}
// a pair of a wall row: where bit V of `solid` is set, the source cell x - c_V is solid and the link
// bounces back, f_V(x) = f*_{opp V}(x) of the previous step (BounceBackWallHalf.h:38-49).  In the AA
// layout that value sits where the other parity's table points: after an odd step in the solid cell's
// slot opp V (the odd table's address), after an even step in the cell's own slot V (the even table's)
template <class S, bool ODD, bool RAW = false>
LBM_D void load_pair_wall(const Params& p, const PairIdx& q, const PairCodec& k, uint32_t solid, F2 (&f)[27]) {
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        if ((solid >> V) & 1u) f[V] = load_dir<S, !ODD, RAW, V>(p, q, k);
        else f[V] = load_dir<S, ODD, RAW, V>(p, q, k);
    });
}
template <class S, bool ODD>
LBM_D void store_pair(const Params& p, const PairIdx& q, const PairCodec& k, const F2 (&f)[27]) {
    using T = typename S::T;
    uint32_t rs = 0;  // stochastic-rounding seed of the pair (FP16)
    if constexpr (S::kind == 2) rs = sr_seed_pair((uint32_t)q.e0, p);
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        T* a = (T*)(ODD ? p.wr_odd[V] : p.wr_even[V]);
        constexpr bool split = ODD && cx(V) != 0;
        const int i0 = cx(V) > 0 ? q.e0 : q.eL, i1 = cx(V) > 0 ? q.eR : q.e1;
        if constexpr (S::kind == 1) {
            if constexpr (split) { a[i0] = f[V].v.x; a[i1] = f[V].v.y; }
            else *(float2*)(a + q.e0) = f[V].v;
        } else {
            const F2 e = lfma(f[V], k.scale, k.nwrs[csq(V)]);
            const __half2 h = half2_sr(e.v, rs + p.sr_off[V]);
            if constexpr (split) { *at32(a, i0) = __low2half(h); *at32(a, i1) = __high2half(h); }
            else *(__half2*)at32(a, q.e0) = h;
        }
    });
}

// bulk pairs on a periodic y or z seam: the neighbour rows wrap, so every access is formed from the
// wrapped row bases R[dy+1][dz+1] and the wrapped x positions xm = x0-1, x2 = x0+2
struct PairRows {
    long long R[3][3];
    int x0, xm, x2;
};
LBM_D void make_pair_rows(const Params& p, int x0, int y, int z, PairRows& w) {
    for (int dz = -1; dz <= 1; dz++)
        for (int dy = -1; dy <= 1; dy++) {
            int yy = y + dy, zz = z + dz;
            if (yy < 0) yy += p.ny; else if (yy >= p.ny) yy -= p.ny;
            if (zz < 0) zz += p.nz; else if (zz >= p.nz) zz -= p.nz;
            w.R[dy + 1][dz + 1] = ((long long)zz * p.ny + yy) * p.nx;
        }
    w.x0 = x0;
    w.xm = x0 == 0 ? p.nx - 1 : x0 - 1;
    w.x2 = x0 + 2 == p.nx ? 0 : x0 + 2;
}
template <class S, bool ODD, bool RAW = false>
LBM_D void load_pair_rows(const Params& p, const PairRows& w, const PairCodec& k, F2 (&f)[27]) {
    using T = typename S::T;
    const T* A = (const T*)p.f;
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        constexpr int slot = ODD ? opp(V) : V;
        const T* a = A + (long long)slot * p.N + (ODD ? w.R[1 - cy(V)][1 - cz(V)] : w.R[1][1]);
        constexpr bool split = ODD && cx(V) != 0;
        // reads of cell x - c_v: c_x = +1 -> (x0-1, x0), c_x = -1 -> (x0+1, x0+2)
        const int i0 = cx(V) > 0 ? w.xm : w.x0 + 1, i1 = cx(V) > 0 ? w.x0 : w.x2;
        if constexpr (S::kind == 1) {
            if constexpr (split) f[V] = F2(__ldg(a + i0), __ldg(a + i1));
            else f[V] = F2(__ldg((const float2*)(a + w.x0)));
        } else {
            float2 t;
            if constexpr (split) t = make_float2(__half2float(__ldg(a + i0)), __half2float(__ldg(a + i1)));
            else t = __half22float2(__ldg((const __half2*)(a + w.x0)));
            if constexpr (RAW) f[V] = F2(t);
            else f[V] = lfma(F2(t), k.inv_scale, k.wr[csq(V)]);
        }
    });
}
template <class S, bool ODD>
LBM_D void store_pair_rows(const Params& p, const PairRows& w, const PairCodec& k, const F2 (&f)[27]) {
    using T = typename S::T;
    T* A = (T*)p.f;
    uint32_t rs = 0;  // stochastic-rounding seed of the pair (FP16), seeded by the pair's first cell
    if constexpr (S::kind == 2) rs = sr_seed_pair((uint32_t)(w.R[1][1] + w.x0), p);
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        constexpr int slot = ODD ? V : opp(V);
        T* a = A + (long long)slot * p.N + (ODD ? w.R[1 + cy(V)][1 + cz(V)] : w.R[1][1]);
        constexpr bool split = ODD && cx(V) != 0;
        // writes to cell x + c_v: c_x = +1 -> (x0+1, x0+2), c_x = -1 -> (x0-1, x0)
        const int i0 = cx(V) > 0 ? w.x0 + 1 : w.xm, i1 = cx(V) > 0 ? w.x2 : w.x0;
        if constexpr (S::kind == 1) {
            if constexpr (split) { a[i0] = f[V].v.x; a[i1] = f[V].v.y; }
            else *(float2*)(a + w.x0) = f[V].v;
        } else {
            const F2 e = lfma(f[V], k.scale, k.nwrs[csq(V)]);
            const __half2 h = half2_sr(e.v, rs + p.sr_off[V]);
            if constexpr (split) { a[i0] = __low2half(h); a[i1] = __high2half(h); }
            else *(__half2*)(a + w.x0) = h;
        }
    });
}

template <class S>
LBM_D PairCodec make_codec(const Params& p) {
    PairCodec k;
    if constexpr (S::kind == 2) {
        k.inv_scale = F2(p.inv_scale);
        k.scale = F2(p.scale);
        k.wr[0] = F2(p.wr[0]); k.wr[1] = F2(p.wr[1]); k.wr[2] = F2(p.wr[7]); k.wr[3] = F2(p.wr[19]);
        k.nwrs[0] = F2(p.nwrs[0]); k.nwrs[1] = F2(p.nwrs[1]); k.nwrs[2] = F2(p.nwrs[7]); k.nwrs[3] = F2(p.nwrs[19]);
    }
    return k;
}
// element indices of the pair whose first cell is element e0 at x = x0 (x seams wrap through eL / eR)
LBM_D PairIdx make_pair_idx(const Params& p, int e0, int x0) {
    PairIdx q;
    q.e0 = e0;
    q.e1 = e0 + 1;
    q.eL = (p.wrap[0] && x0 == 0) ? e0 + p.nx : e0;
    q.eR = (p.wrap[0] && x0 + 2 == p.nx) ? q.e1 - p.nx : q.e1;
    return q;
}

// the collision the packed path runs for the collision policy (the combined one packs only pairs of
// reference-flag-1 cells, which both take the 2015 branch), and whether it takes its moments from the
// raw FP16 deviations (FP16 + cumulant-2015)
template <int COLL> LBM_HD constexpr int packed_coll() { return COLL == 3 ? 1 : COLL; }
template <class S, int COLL> LBM_HD constexpr bool packed_raw() { return S::kind == 2 && packed_coll<COLL>() == 1; }

// one packed pair of bulk cells in a row off the periodic y/z seams: every access is a per-direction
// base address plus the element index.  CLOS 2: the learned closure's steps between network evaluations
// (the pair's kept nu_t, Params::nut, fetched before the populations)
template <class S, int COLL, int CLOS, bool ODD>
LBM_D void step_pair_plain(const Params& p, int e0, int x0) {
    constexpr int PC = packed_coll<COLL>();
    constexpr bool RAW = packed_raw<S, COLL>();
    const PairCodec k = make_codec<S>(p);
    const PairIdx q = make_pair_idx(p, e0, x0);
    float2 kept = make_float2(-1.f, -1.f);
    if constexpr (CLOS == 2) kept = __half22float2(__ldg((const __half2*)(p.nut + e0)));
    // FP16 storage: the pair's two class bytes in one 16-bit load ahead of the populations (1 B per
    // cell), checked against the packed kind after the stores.  Measured at 512x256x256: the FP16
    // Smagorinsky step 49.6 GLUPS without the load, 51.3 with the check after the stores, 50.5 after
    // the collision, 49.3 before it; with the early load the long-scoreboard stalls per issue fall from
    // 4.7 to 3.4 (even steps, ncu) and the even kernel no longer spills.  SRT 38.1 -> 40.1, combined
    // 46.6 -> 48.3; cumulant-2017 36.3 -> 35.9, so it keeps no check (nor does the kept-rate step, whose
    // kept nu_t is such an early load already)
    constexpr bool CHECK = S::kind == 2 && CLOS != 2 && COLL != 2;
    uint32_t cls2 = 0;
    if constexpr (CHECK) cls2 = __ldg((const uint16_t*)(p.cls + e0));
    F2 f[27];
    load_pair<S, ODD, RAW>(p, q, k, f);
    collide_pair<PC, CLOS, RAW>(p, f, e0, kept);
    store_pair<S, ODD>(p, q, k, f);
    if constexpr (CHECK) {
        constexpr uint32_t keep = COLL == 3 ? 0xffffu : (uint32_t)(uint8_t)~BIT_REFBULK * 0x0101u;
        constexpr uint32_t want = (COLL == 3 ? (uint32_t)(CLS_BULK | BIT_REFBULK) : (uint32_t)CLS_BULK) * 0x0101u;
        if ((cls2 & keep) != want) *p.err = DEV_ERR_ROW_LIST;
    }
}

// one x-pair (x0 even): packed path for two bulk cells, else the per-cell path for each
template <class S, int COLL, int CLOS, bool ODD>
LBM_D void step_pair(const Params& p, int x0, int y, int z) {
    static_assert(S::kind != 0, "packed pairs are FP32 arithmetic");
    const bool two = x0 + 1 < p.nx;
    const unsigned idx0 = (unsigned)x0 + (unsigned)p.nx * ((unsigned)y + (unsigned)p.ny * (unsigned)z);
    constexpr uint8_t keep = COLL == 3 ? (uint8_t)0xff : (uint8_t)~BIT_REFBULK;
    constexpr uint8_t want = COLL == 3 ? (uint8_t)(CLS_BULK | BIT_REFBULK) : (uint8_t)CLS_BULK;
    constexpr int PC = packed_coll<COLL>();
    constexpr bool RAW = packed_raw<S, COLL>();
    const uint8_t f0 = p.cls[idx0] & keep;
    const uint8_t f1 = two ? (p.cls[idx0 + 1] & keep) : (uint8_t)0;
    const bool pair = two && f0 == want && f1 == want && (p.nx & 1) == 0;
    if (!pair) {
        step_cell_call<S, COLL, CLOS, ODD>(p, x0, y, z);
        if (two) step_cell_call<S, COLL, CLOS, ODD>(p, x0 + 1, y, z);
        return;
    }
    // rows on a periodic y or z seam (uniform per block) form their addresses from wrapped rows;
    // all other rows use the per-direction base addresses (x seams wrap through eL / eR)
    const bool yz_seam = (p.wrap[1] && (y == 0 || y == p.ny - 1)) || (p.wrap[2] && (z == 0 || z == p.nz - 1));
    if (!yz_seam) {
        step_pair_plain<S, COLL, CLOS, ODD>(p, (int)idx0, x0);
    } else {
        const PairCodec k = make_codec<S>(p);
        F2 f[27];
        PairRows w;
        make_pair_rows(p, x0, y, z, w);
        load_pair_rows<S, ODD, RAW>(p, w, k, f);
        collide_pair<PC, CLOS, RAW>(p, f, idx0);
        store_pair_rows<S, ODD>(p, w, k, f);
    }
}

// minimum resident CTAs per SM requested from the register allocator, per collision (0: no request),
// measured on a GB300 on the 512x256x256 channel (GLUPS, FP16-deviation / FP32 storage):
//   cumulant-2015: 6 (at most 85 registers, a few spilled to L1): 40.0 / 30.9, against 36.7 / 30.2 with
//                  no request (128 registers); 5, 7 and 8 slower;
//   SRT:           4 (128 registers): 31.8 / 26.7, against 22.9 / 21.9 with none (250 registers),
//                  29.9 / 26.6 at 3, 23.2 / 18.9 at 5, 16.2 / 13.8 at 6 (1.8 KB spilled);
//   cumulant-2017: 4: 29.5 / 28.3, against 26.9 / 24.8 with none (166 registers), 29.5 / 27.9 at 5,
//                  26.8 / 23.6 at 6.
#ifndef LBM_STEP2_MIN_BLOCKS
#define LBM_STEP2_MIN_BLOCKS 6
#endif
#ifndef LBM_STEP2_MIN_BLOCKS_SRT
#define LBM_STEP2_MIN_BLOCKS_SRT 4
#endif
#ifndef LBM_STEP2_MIN_BLOCKS_CUM17
#define LBM_STEP2_MIN_BLOCKS_CUM17 4
#endif
#ifndef LBM_STEP2_MIN_BLOCKS_COMBINED
#define LBM_STEP2_MIN_BLOCKS_COMBINED LBM_STEP2_MIN_BLOCKS
#endif
constexpr int step2_min_blocks(int coll) {
    return coll == 1 ? LBM_STEP2_MIN_BLOCKS
         : coll == 0 ? LBM_STEP2_MIN_BLOCKS_SRT
         : coll == 2 ? LBM_STEP2_MIN_BLOCKS_CUM17
                     : LBM_STEP2_MIN_BLOCKS_COMBINED;
}
template <class S, int COLL, int CLOS, bool ODD>
__global__ void __launch_bounds__(128, step2_min_blocks(COLL)) k_step2(Params p) {
    const int x0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (x0 >= p.nx) return;
    step_pair<S, COLL, CLOS, ODD>(p, x0, blockIdx.y, blockIdx.z);
}

// ---- the step split by rows ------------------------------------------------------------------------
// Set-up lists the plain rows (every cell a bulk fluid cell of the packed path, the row off the periodic
// y/z seams, nx even) and the remaining rows.  k_step2_plain runs only the packed pair path over the
// plain rows: no class dispatch (FP16 loads the class bytes only to check them after the stores), no
// per-cell fallback, so the register allocation is that of the packed path alone.  k_step2_list runs the general pair step over the remaining rows.  Every population slot
// is read and written by one thread only within a step (the AA argument), so running the two sets of
// threads as two launches gives the same result as one launch over the lattice.
// Grid: x = block of 128 x-pairs in the row, y and z = row in the list (rows_grid), so the blocks of a
// row are adjacent and neighbouring rows run together, as in the one-launch grid.
// resident CTAs per SM for the plain-row kernel (cumulant-2015), measured at 512x256x256 FP16: 7 (72
// registers, 16 bytes spilled on odd steps) 42.5 GLUPS against 40.9 at 6 (80 registers) and less at 5
#ifndef LBM_PLAIN_MIN_BLOCKS
#define LBM_PLAIN_MIN_BLOCKS 7
#endif
#ifndef LBM_PLAIN_MIN_BLOCKS_SRT
#define LBM_PLAIN_MIN_BLOCKS_SRT 4
#endif
#ifndef LBM_PLAIN_MIN_BLOCKS_CUM17
#define LBM_PLAIN_MIN_BLOCKS_CUM17 4
#endif
// FP32 storage (HBM-bound at 80 registers, no spill): as k_step2
#ifndef LBM_PLAIN_MIN_BLOCKS_F32
#define LBM_PLAIN_MIN_BLOCKS_F32 LBM_STEP2_MIN_BLOCKS
#endif
constexpr int plain_min_blocks(int coll, int kind = 2) {
    return coll == 0 ? LBM_PLAIN_MIN_BLOCKS_SRT : coll == 2 ? LBM_PLAIN_MIN_BLOCKS_CUM17
         : kind == 1 ? LBM_PLAIN_MIN_BLOCKS_F32 : LBM_PLAIN_MIN_BLOCKS;
}
// blocks of 128 x-pairs per row: blockIdx.x = block within the row, list entry = blockIdx.y + gridDim.y
// blockIdx.z (rows_grid); returns false for the tail blocks past the list
LBM_D bool row_block(const int32_t* rows, int n, int& r, int& x0) {
    const int e = (int)(blockIdx.y + gridDim.y * blockIdx.z);
    if (e >= n) return false;
    r = rows[e];
    x0 = 2 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    return true;
}
template <class S, int COLL, int CLOS, bool ODD>
__global__ void __launch_bounds__(128, plain_min_blocks(COLL, S::kind)) k_step2_plain(Params p, const int32_t* rows, int n) {
    int r, x0;
    if (!row_block(rows, n, r, x0) || x0 >= p.nx) return;
    step_pair_plain<S, COLL, CLOS, ODD>(p, r * p.nx + x0, x0);
}
// rows beside a flat wall (set-up lists them with the row's solid-source mask): every cell an edge cell
// whose solid neighbours lie at the same offsets, so the whole row takes the packed pair path with the
// bounce-back links read through the other parity's address table (load_pair_wall)
template <class S, int COLL, int CLOS, bool ODD>
__global__ void __launch_bounds__(128, plain_min_blocks(COLL, S::kind)) k_step2_wall(Params p, const int32_t* rows,
                                                                                   const uint32_t* solid, int n) {
    int r, x0;
    if (!row_block(rows, n, r, x0) || x0 >= p.nx) return;
    // at m = 0 every cell reads its own initial slots (there is no previous post-collision state to
    // bounce back, and the solid cells' slots hold zeros): the gather rule of the per-cell path
    const uint32_t m = p.m == 0 ? 0u : solid[blockIdx.y + gridDim.y * blockIdx.z];
    constexpr int PC = packed_coll<COLL>();
    constexpr bool RAW = packed_raw<S, COLL>();
    const int e0 = r * p.nx + x0;
    const PairCodec k = make_codec<S>(p);
    const PairIdx q = make_pair_idx(p, e0, x0);
    F2 f[27];
    load_pair_wall<S, ODD, RAW>(p, q, k, m, f);
    collide_pair<PC, CLOS, RAW>(p, f, e0);
    store_pair<S, ODD>(p, q, k, f);
}
template <class S, int COLL, int CLOS, bool ODD>
__global__ void __launch_bounds__(128, step2_min_blocks(COLL)) k_step2_list(Params p, const int32_t* rows, int n) {
    int r, x0;
    if (!row_block(rows, n, r, x0) || x0 >= p.nx) return;
    step_pair<S, COLL, CLOS, ODD>(p, x0, r % p.ny, r / p.ny);
}

}  // namespace lbm
