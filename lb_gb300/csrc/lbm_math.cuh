// lbm_math.cuh - per-cell collision mathematics, generic over the "lane" type:
//   float / double : one cell per thread;
//   F2             : two cells per thread in packed FP32 (FADD2 / FMUL2 / FFMA2 on sm_100+),
//                    one issue slot for two cells' worth of arithmetic.
// Every function takes populations in the reference's velocity order (D3Q27.h:81-111).
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

namespace lbm {

#ifndef LBM_HD
#define LBM_HD __host__ __device__ __forceinline__
#define LBM_D __device__ __forceinline__
#endif

// ---- velocity set ---------------------------------------------------------------------------------
LBM_HD constexpr int cx(int v) {
    constexpr int t[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, -1, 1, 0, 0, -1, 1, 0, 0, -1, 1, -1, 1, 1, -1, -1, 1};
    return t[v];
}
LBM_HD constexpr int cy(int v) {
    constexpr int t[27] = {0, 0, 0, 0, 0, -1, 1, 0, 0, 0, 0, -1, 1, 1, -1, 1, -1, 1, -1, 1, -1, -1, 1, -1, 1, -1, 1};
    return t[v];
}
LBM_HD constexpr int cz(int v) {
    constexpr int t[27] = {0, 0, 0, -1, 1, 0, 0, -1, 1, 1, -1, 0, 0, -1, 1, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, -1, 1};
    return t[v];
}
LBM_HD constexpr int opp(int v) { return v == 0 ? 0 : ((v & 1) ? v + 1 : v - 1); }
LBM_HD constexpr int csq(int v) { return cx(v) * cx(v) + cy(v) * cy(v) + cz(v) * cz(v); }
LBM_HD constexpr double wgt(int v) {
    return csq(v) == 0 ? 8.0 / 27.0 : csq(v) == 1 ? 2.0 / 27.0 : csq(v) == 2 ? 1.0 / 54.0 : 1.0 / 216.0;
}
// direction index of the velocity (x, y, z) in {-1,0,1}^3
LBM_HD constexpr int vid(int x, int y, int z) {
    for (int v = 0; v < 27; v++)
        if (cx(v) == x && cy(v) == y && cz(v) == z) return v;
    return -1;
}

template <int I, int N, class F>
LBM_D void sfor(F&& f) {
    if constexpr (I < N) {
        f(std::integral_constant<int, I>{});
        sfor<I + 1, N>(f);
    }
}

// ---- lane types ---------------------------------------------------------------------------------
struct F2 {
    float2 v;
    LBM_D F2() {}
    LBM_D F2(float s) : v(make_float2(s, s)) {}
    LBM_D F2(double s) : v(make_float2((float)s, (float)s)) {}
    LBM_D F2(int s) : v(make_float2((float)s, (float)s)) {}
    LBM_D F2(float a, float b) : v(make_float2(a, b)) {}
    LBM_D explicit F2(float2 a) : v(a) {}
};
// subtraction and negation as one packed FFMA2 / FMUL2 with the constant pair (-1, -1):
// b * (-1) is exact, so a - b rounds once, as FADD would
LBM_D F2 operator+(F2 a, F2 b) { return F2(__fadd2_rn(a.v, b.v)); }
LBM_D F2 operator-(F2 a) { return F2(__fmul2_rn(a.v, make_float2(-1.0f, -1.0f))); }
LBM_D F2 operator-(F2 a, F2 b) { return F2(__ffma2_rn(b.v, make_float2(-1.0f, -1.0f), a.v)); }
LBM_D F2 operator*(F2 a, F2 b) { return F2(__fmul2_rn(a.v, b.v)); }
LBM_D F2& operator+=(F2& a, F2 b) { a = a + b; return a; }
LBM_D F2& operator-=(F2& a, F2 b) { a = a - b; return a; }

LBM_D float lfma(float a, float b, float c) { return fmaf(a, b, c); }
LBM_D double lfma(double a, double b, double c) { return fma(a, b, c); }
LBM_D F2 lfma(F2 a, F2 b, F2 c) { return F2(__ffma2_rn(a.v, b.v, c.v)); }

// reciprocal and square root: FP32 uses the SFU approximations (the reference builds with
// -use_fast_math, 3D/simulation/src/config/config.mk:37); FP64 stays IEEE
LBM_D float rcp(float x) { return __fdividef(1.0f, x); }
LBM_D double rcp(double x) { return 1.0 / x; }
LBM_D F2 rcp(F2 x) { return F2(__fdividef(1.0f, x.v.x), __fdividef(1.0f, x.v.y)); }
LBM_D float sqrt_pos(float x) { x = fmaxf(x, 1e-30f); return x * rsqrtf(x); }
LBM_D double sqrt_pos(double x) { return sqrt(x); }
LBM_D F2 sqrt_pos(F2 x) { return F2(sqrt_pos(x.v.x), sqrt_pos(x.v.y)); }

// c . u with the zero components skipped at compile time
template <int V, class L>
LBM_D L cdotu(L ux, L uy, L uz) {
    L r = (L)0.0f;
    bool any = false;
    auto add = [&](int c, L u) {
        if (c == 0) return;
        if (!any) { r = c > 0 ? u : -u; any = true; }
        else r = c > 0 ? r + u : r - u;
    };
    add(cx(V), ux);
    add(cy(V), uy);
    add(cz(V), uz);
    return r;
}

// ---- moments up to second order ------------------------------------------------------------------
// z pairs within each (c_x, c_y) column, then y, then x: the forward half of the chimera transform
// (G2015 eq. 43-45) evaluated at u = 0, i.e. raw moments
template <class L>
struct Mom {
    L rho, jx, jy, jz, Mxx, Myy, Mzz, Mxy, Mxz, Myz;
};
template <class L>
LBM_D Mom<L> raw_moments(const L (&f)[27]) {
    L s0[3][3], sb[3][3], sa[3][3];
    sfor<0, 3>([&](auto xc) {
        constexpr int X = decltype(xc)::value;
        sfor<0, 3>([&](auto yc) {
            constexpr int Y = decltype(yc)::value;
            const L fm = f[vid(X - 1, Y - 1, -1)], fz = f[vid(X - 1, Y - 1, 0)], fp = f[vid(X - 1, Y - 1, 1)];
            sa[X][Y] = fp + fm;   // sum f c_z^2
            sb[X][Y] = fp - fm;   // sum f c_z
            s0[X][Y] = sa[X][Y] + fz;
        });
    });
    L T0[3], Ty[3], Tyy[3], Tz[3], Tyz[3], Tzz[3];
    sfor<0, 3>([&](auto xc) {
        constexpr int X = decltype(xc)::value;
        Tyy[X] = s0[X][2] + s0[X][0];
        T0[X] = Tyy[X] + s0[X][1];
        Ty[X] = s0[X][2] - s0[X][0];
        Tz[X] = (sb[X][2] + sb[X][0]) + sb[X][1];
        Tyz[X] = sb[X][2] - sb[X][0];
        Tzz[X] = (sa[X][2] + sa[X][0]) + sa[X][1];
    });
    Mom<L> m;
    m.Mxx = T0[2] + T0[0];
    m.rho = m.Mxx + T0[1];
    m.jx = T0[2] - T0[0];
    m.jy = (Ty[2] + Ty[0]) + Ty[1];
    m.Mxy = Ty[2] - Ty[0];
    m.Myy = (Tyy[2] + Tyy[0]) + Tyy[1];
    m.jz = (Tz[2] + Tz[0]) + Tz[1];
    m.Mxz = Tz[2] - Tz[0];
    m.Myz = (Tyz[2] + Tyz[0]) + Tyz[1];
    m.Mzz = (Tzz[2] + Tzz[0]) + Tzz[1];
    return m;
}

// ---- relaxation rate ----------------------------------------------------------------------------
// Smagorinsky (OmegaLES.h:312-357): Pi = sum c c (f - f_eq) = M - rho (u u + I/3),
// tau_LES = tau/2 + sqrt(tau^2 + 18 CLES |Pi| / rho)/2
template <class L>
LBM_D L omega_smagorinsky(L tau, L cles18, L rho, L ri, L ux, L uy, L uz, const Mom<L>& m) {
    const L third = rho * (L)(1.0 / 3.0);
    const L rux = rho * ux, ruy = rho * uy, ruz = rho * uz;
    const L pxx = lfma(-rux, ux, m.Mxx - third), pyy = lfma(-ruy, uy, m.Myy - third), pzz = lfma(-ruz, uz, m.Mzz - third);
    const L pxy = lfma(-rux, uy, m.Mxy), pxz = lfma(-rux, uz, m.Mxz), pyz = lfma(-ruy, uz, m.Myz);
    const L off = lfma(pxy, pxy, lfma(pxz, pxz, pyz * pyz));
    const L PI2 = lfma(pxx, pxx, lfma(pyy, pyy, lfma(pzz, pzz, off + off)));
    const L PI = sqrt_pos(PI2);
    const L tles = lfma(tau, (L)0.5f, (L)0.5f * sqrt_pos(lfma(tau, tau, cles18 * ri * PI)));
    return rcp(tles);
}

// ---- SRT (CollisionSRTTurbulent.h:386-391) --------------------------------------------------------
template <class L>
LBM_D void collide_srt(L (&f)[27], L rho, L ux, L uy, L uz, L om) {
    const L u2 = lfma(ux, ux, lfma(uy, uy, uz * uz));
    const L base = lfma((L)-1.5f, u2, (L)1.0f);
    const L wr0 = rho * (L)(8.0 / 27.0), wr1 = rho * (L)(2.0 / 27.0), wr2 = rho * (L)(1.0 / 54.0),
            wr3 = rho * (L)(1.0 / 216.0);
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        const L wr = csq(V) == 0 ? wr0 : csq(V) == 1 ? wr1 : csq(V) == 2 ? wr2 : wr3;
        L e;
        if constexpr (V == 0) {
            e = base;
        } else {
            const L cu = cdotu<V>(ux, uy, uz);
            e = lfma(cu, lfma((L)4.5f, cu, (L)3.0f), base);  // 1 + 3cu + 4.5cu^2 - 1.5u^2
        }
        const L feq = wr * e;
        f[V] = lfma(om, feq - f[V], f[V]);  // f - om (f - feq)
    });
}
// Guo forcing term added after collide_srt (no reference counterpart)
template <class L>
LBM_D void srt_force(L (&f)[27], L ux, L uy, L uz, L om, L Fx, L Fy, L Fz) {
    const L gf = lfma((L)-0.5f, om, (L)1.0f);
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        const L cu = V == 0 ? (L)0.0f : cdotu<V>(ux, uy, uz);
        const L s = ((L)3.0f * ((L)(float)cx(V) - ux) + (L)9.0f * cu * (L)(float)cx(V)) * Fx +
                    ((L)3.0f * ((L)(float)cy(V) - uy) + (L)9.0f * cu * (L)(float)cy(V)) * Fy +
                    ((L)3.0f * ((L)(float)cz(V) - uz) + (L)9.0f * cu * (L)(float)cz(V)) * Fz;
        f[V] = lfma(gf * (L)wgt(V), s, f[V]);
    });
}

// ---- cumulant collision, Geier 2015 with omega_2..omega_10 = 1 -----------------------------------
// Same operator as CollisionCumD3Q27Turbulent2015.h:80-485, written in closed form: with all higher
// relaxation rates equal to one, every post-collision cumulant above second order is zero, so only
// the second-order central moments are needed from the forward transform and the backward
// (chimera, G2015 eq. 88-96) transform takes the products of eq. 81-84.
//
// backward triplet: central moments (k0, k1, k2) along one axis -> populations (m, 0, p):
//   m = (k0 (u^2-u) + k1 (2u-1) + k2) / 2,  p = m + k0 u + k1,  z = k0 (1-u^2) - 2u k1 - k2
template <class L>
struct Axis {
    L u, A, B, C, m2u;  // u, (u^2-u)/2, u-1/2, 1-u^2, -2u
};
template <class L>
LBM_D Axis<L> make_axis(L u, L uu) {
    Axis<L> a;
    a.u = u;
    a.A = (L)0.5f * (uu - u);
    a.B = u - (L)0.5f;
    a.C = (L)1.0f - uu;
    a.m2u = (L)-2.0f * u;
    return a;
}
template <class L>
LBM_D void tri(L k0, L k1, L k2, const Axis<L>& a, L& m, L& z, L& p) {
    m = lfma(k0, a.A, lfma(k1, a.B, (L)0.5f * k2));
    p = m + lfma(k0, a.u, k1);
    z = lfma(k0, a.C, lfma(a.m2u, k1, -k2));
}
template <class L>
LBM_D void tri_k1zero(L k0, L k2, const Axis<L>& a, L& m, L& z, L& p) {  // k1 = 0
    m = lfma(k0, a.A, (L)0.5f * k2);
    p = lfma(k0, a.u, m);
    z = lfma(k0, a.C, -k2);
}
template <class L>
LBM_D void tri_k2zero(L k0, L k1, const Axis<L>& a, L& m, L& z, L& p) {  // k2 = 0
    m = lfma(k0, a.A, k1 * a.B);
    p = m + lfma(k0, a.u, k1);
    z = lfma(k0, a.C, a.m2u * k1);
}
template <class L>
LBM_D void tri_k1only(L k1, const Axis<L>& a, L& m, L& z, L& p) {  // k0 = k2 = 0
    m = k1 * a.B;
    p = m + k1;
    z = a.m2u * k1;
}

template <class L>
LBM_D void collide_cum15(L (&f)[27], L rho, L ri, L ux, L uy, L uz, L om, const Mom<L>& mm) {
    const L uxx = ux * ux, uyy = uy * uy, uzz = uz * uz;
    // central moments; k_100 = j_x - rho u_x carries the half-force shift (G2015 eq. 85-87)
    const L rux = rho * ux, ruy = rho * uy, ruz = rho * uz;
    const L q100 = rux - mm.jx, q010 = ruy - mm.jy, q001 = ruz - mm.jz;  // -k_100, ...
    const L C200 = lfma(ux, rux - mm.jx - mm.jx, mm.Mxx);               // Mxx - 2 ux jx + rho ux^2
    const L C020 = lfma(uy, ruy - mm.jy - mm.jy, mm.Myy);
    const L C002 = lfma(uz, ruz - mm.jz - mm.jz, mm.Mzz);
    const L C110 = lfma(ux, ruy - mm.jy, lfma(-uy, mm.jx, mm.Mxy));      // Mxy - ux jy - uy jx + rho ux uy
    const L C101 = lfma(ux, ruz - mm.jz, lfma(-uz, mm.jx, mm.Mxz));
    const L C011 = lfma(uy, ruz - mm.jz, lfma(-uz, mm.jy, mm.Myz));
    // relaxation, G2015 eq. 55-63 with omega_2 = 1
    const L h = (L)0.5f * ri;
    const L d20 = C200 - C020, d02 = C200 - C002;
    const L Dxu = -h * lfma(om, d20 + d02, C200 + C020 + C002 - rho);
    const L t3oh = (L)3.0f * om * h;
    const L Dyv = lfma(t3oh, d20, Dxu);
    const L Dzw = lfma(t3oh, d02, Dxu);
    const L o1 = (L)1.0f - om;
    const L a = rho * lfma((L)-1.5f, om, (L)3.0f);  // 3 rho (1 - om/2)
    const L xD = uxx * Dxu, yD = uyy * Dyv, zD = uzz * Dzw;
    const L E61 = lfma(o1, d20, a * (yD - xD));
    const L E64 = lfma(o1, d02, a * (zD - xD));
    const L E65 = lfma((L)-1.5f * rho, xD + yD + zD, rho);
    const L t3 = (L)(1.0 / 3.0);
    const L s200 = (E61 + E64 + E65) * t3;
    const L s020 = lfma((L)-2.0f, E61, E64 + E65) * t3;
    const L s002 = lfma((L)-2.0f, E64, E61 + E65) * t3;
    const L s110 = o1 * C110, s101 = o1 * C101, s011 = o1 * C011;
    // post-collision central moments (G2015 eq. 81-84; third order and relaxed higher cumulants zero)
    const L p1 = s101 * s110, p2 = s110 * s011, p3 = s011 * s101;
    const L q211 = lfma(s200, s011, p1 + p1) * ri;
    const L q121 = lfma(s020, s101, p2 + p2) * ri;
    const L q112 = lfma(s002, s110, p3 + p3) * ri;
    const L q220 = lfma(s020, s200, (L)2.0f * s110 * s110) * ri;
    const L q022 = lfma(s002, s020, (L)2.0f * s011 * s011) * ri;
    const L q202 = lfma(s200, s002, (L)2.0f * s101 * s101) * ri;
    const L sum4 = lfma(s011, q211, lfma(s101, q121, s110 * q112));
    const L first = lfma(s200, q022, lfma(s020, q202, lfma(s002, q220, (L)4.0f * sum4)));
    const L sq4 = lfma(s101 * s101, s020, lfma(s011 * s011, s200, s110 * s110 * s002));
    const L second = lfma((L)16.0f * s110, s101 * s011, lfma((L)4.0f, sq4, (L)2.0f * s200 * s020 * s002));
    const L q222 = (first - second * ri) * ri;
    // backward chimera transform: x pass (9 triplets over (oy, oz)), then y, then z
    const Axis<L> ax = make_axis(ux, uxx), ay = make_axis(uy, uyy), az = make_axis(uz, uzz);
    L g[3][3][3];  // [sx][oy][oz]
    tri(rho, q100, s200, ax, g[0][0][0], g[1][0][0], g[2][0][0]);
    tri_k2zero(q001, s101, ax, g[0][0][1], g[1][0][1], g[2][0][1]);
    tri_k1zero(s002, q202, ax, g[0][0][2], g[1][0][2], g[2][0][2]);
    tri_k2zero(q010, s110, ax, g[0][1][0], g[1][1][0], g[2][1][0]);
    tri_k1zero(s011, q211, ax, g[0][1][1], g[1][1][1], g[2][1][1]);
    tri_k1only(q112, ax, g[0][1][2], g[1][1][2], g[2][1][2]);
    tri_k1zero(s020, q220, ax, g[0][2][0], g[1][2][0], g[2][2][0]);
    tri_k1only(q121, ax, g[0][2][1], g[1][2][1], g[2][2][1]);
    tri_k1zero(q022, q222, ax, g[0][2][2], g[1][2][2], g[2][2][2]);
    L hh[3][3][3];  // [sx][sy][oz]
    sfor<0, 3>([&](auto sc) {
        constexpr int SX = decltype(sc)::value;
        sfor<0, 3>([&](auto oc) {
            constexpr int OZ = decltype(oc)::value;
            tri(g[SX][0][OZ], g[SX][1][OZ], g[SX][2][OZ], ay, hh[SX][0][OZ], hh[SX][1][OZ], hh[SX][2][OZ]);
        });
    });
    sfor<0, 3>([&](auto sc) {
        constexpr int SX = decltype(sc)::value;
        sfor<0, 3>([&](auto yc) {
            constexpr int SY = decltype(yc)::value;
            L m, z, p;
            tri(hh[SX][SY][0], hh[SX][SY][1], hh[SX][SY][2], az, m, z, p);
            f[vid(SX - 1, SY - 1, -1)] = m;
            f[vid(SX - 1, SY - 1, 0)] = z;
            f[vid(SX - 1, SY - 1, 1)] = p;
        });
    });
}

}  // namespace lbm
