// lbm_math.cuh - per-cell collision mathematics, generic over the "lane" type:
//   float / double : one cell per thread;
//   F2             : two cells per thread in packed FP32 (FADD2 / FMUL2 / FFMA2 on sm_100+),
//                    one issue slot for two cells' worth of arithmetic.
// Every function takes populations in the reference's velocity order (D3Q27.h:81-111).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

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

// ---- conversions between FP32 and FP64 on the integer pipe ---------------------------------------
// GB300 executes FP64 instructions, conversions included, at about one lane per cycle per SM, so the
// read and set-up kernels convert with integer operations: exact for every finite FP32 value, round to
// nearest even for FP64 values in the FP32 normal range; zero keeps its sign; anything else (FP32
// subnormal results, overflow, NaN) falls back to the hardware conversion.
LBM_D double f2d(float x) {
    const uint32_t b = __float_as_uint(x), e = (b >> 23) & 0xFFu;
    if ((b & 0x7FFFFFFFu) == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);  // signed zero
    if (e == 0u || e == 0xFFu) return (double)x;  // subnormal, inf, NaN: exact either way
    const uint32_t hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7FFFFFu) >> 3);
    const uint32_t lo = b << 29;
    return __hiloint2double((int)hi, (int)lo);
}
LBM_D float d2f(double x) {
    const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
    const uint32_t e = (hi >> 20) & 0x7FFu;
    if (e < 897u || e > 1149u) {  // zero or outside the FP32 normal range (2^-126 .. 2^127)
        if (e == 0u && (hi & 0xFFFFFu) == 0u && lo == 0u) return __uint_as_float(hi & 0x80000000u);
        return __double2float_rn(x);
    }
    // 23 kept mantissa bits, 29 dropped; round half to even; a carry moves into the exponent
    uint32_t m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const uint32_t rem = lo & 0x1FFFFFFFu;
    uint32_t b = (hi & 0x80000000u) | (((e - 896u) << 23) + m);
    if (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) b += 1u;
    return __uint_as_float(b);
}

// compensated FP32 sum (a float-float pair): TwoSum keeps each addition's rounding error in lo, so the
// pair carries about 48 bits; used for the per-thread and per-warp partial sums of the reductions in
// place of FP64 arithmetic
struct FSum {
    float hi, lo;
};
LBM_D void fsum_add(FSum& s, float x) {
    const float t = s.hi + x;
    const float bp = t - s.hi;
    s.lo += (s.hi - (t - bp)) + (x - bp);
    s.hi = t;
}
LBM_D void fsum_merge(FSum& s, const FSum& o) {
    fsum_add(s, o.hi);
    s.lo += o.lo;
}

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
// Smagorinsky (OmegaLES.h:84-129): Pi = sum c c (f - f_eq) = M - rho (u u + I/3),
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

// ---- SRT (CollisionSRTTurbulent.h:63-68) --------------------------------------------------------
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
// the three outputs add up to k0 (m + z + p = k0 for any u), so z = k0 - (m + p): two operations
// instead of three
template <class L>
LBM_D void tri(L k0, L k1, L k2, const Axis<L>& a, L& m, L& z, L& p) {
    m = lfma(k0, a.A, lfma(k1, a.B, (L)0.5f * k2));
    p = m + lfma(k0, a.u, k1);
    z = k0 - (m + p);
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


// ---- cumulant collision with the 2017 parametrisation (CollisionCumD3Q27Turbulent2017.h:241-376) -----
// Full forward chimera transform (G2015 eq. 43-45) to the 27 central moments, cumulants (eq. 47-54),
// relaxation with omega_1 local and omega_2 = 1: third-order rates from G2017 eq. 14-16 limited by
// |C| / (rho lambda + |C|), lambda = 0.01 (section 7); fourth-order cumulants driven by the velocity
// gradients through A and B (G2017 eq. 43-48); omega_6..10 = 1; then eq. 81-87 and the backward
// transform.  The three reference defects (the omega_210 limiters reading C120 +- C102, the bulk part
// of Dxu subtracting rho - 1 instead of k000, and eq. 44 driven by Dxu + Dyv - 2 Dzw, which breaks the
// operator's invariance under axis relabelling) are corrected here; the oracle reproduces them on request.
LBM_D float labs_(float x) { return fabsf(x); }
LBM_D double labs_(double x) { return fabs(x); }
LBM_D F2 labs_(F2 x) { return F2(fabsf(x.v.x), fabsf(x.v.y)); }

// forward triplet: populations (m, z, p) along one axis -> central moments (k0, k1, k2)
template <class L>
LBM_D void tri_fwd(L m, L z, L p, L u, L& k0, L& k1, L& k2) {
    const L s = p + m, d = p - m;
    k0 = s + z;
    k1 = lfma(-u, k0, d);
    k2 = lfma(u, lfma(u, k0, (L)-2.0f * d), s);  // s - 2u d + u^2 k0
}

template <class L>
LBM_D void collide_cum17(L (&f)[27], L rho, L ri, L ux, L uy, L uz, L om) {
    L k[3][3][3];
    // z pass, y pass, x pass (indices: slot c+1 before the pass, moment order after it)
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const int vm = vid(a - 1, b - 1, -1), vz = vid(a - 1, b - 1, 0), vp = vid(a - 1, b - 1, 1);
            tri_fwd(f[vm], f[vz], f[vp], uz, k[a][b][0], k[a][b][1], k[a][b][2]);
        }
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            L k0, k1, k2;
            tri_fwd(k[a][0][c], k[a][1][c], k[a][2][c], uy, k0, k1, k2);
            k[a][0][c] = k0; k[a][1][c] = k1; k[a][2][c] = k2;
        }
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            L k0, k1, k2;
            tri_fwd(k[0][b][c], k[1][b][c], k[2][b][c], ux, k0, k1, k2);
            k[0][b][c] = k0; k[1][b][c] = k1; k[2][b][c] = k2;
        }
    const L one = (L)1.0f, two = (L)2.0f, four = (L)4.0f, half = (L)0.5f, third = (L)(1.0 / 3.0);
    // cumulants of order 4 to 6 (G2015 eq. 51-54); orders 2 and 3 equal the central moments
    const L K000 = k[0][0][0], K100 = k[1][0][0], K010 = k[0][1][0], K001 = k[0][0][1];
    const L C110 = k[1][1][0], C101 = k[1][0][1], C011 = k[0][1][1];
    const L C200 = k[2][0][0], C020 = k[0][2][0], C002 = k[0][0][2];
    const L C120 = k[1][2][0], C102 = k[1][0][2], C210 = k[2][1][0], C012 = k[0][1][2], C201 = k[2][0][1],
            C021 = k[0][2][1], C111 = k[1][1][1];
    const L C211 = k[2][1][1] - lfma(C200, C011, two * C101 * C110) * ri;
    const L C121 = k[1][2][1] - lfma(C020, C101, two * C110 * C011) * ri;
    const L C112 = k[1][1][2] - lfma(C002, C110, two * C011 * C101) * ri;
    const L C220 = k[2][2][0] - lfma(C020, C200, two * C110 * C110) * ri;
    const L C022 = k[0][2][2] - lfma(C002, C020, two * C011 * C011) * ri;
    const L C202 = k[2][0][2] - lfma(C200, C002, two * C101 * C101) * ri;
    const L C122 = k[1][2][2] - (lfma(C020, C102, lfma(C002, C120, four * C011 * C111)) +
                                 two * lfma(C110, C012, C101 * C021)) * ri;
    const L C212 = k[2][1][2] - (lfma(C002, C210, lfma(C200, C012, four * C101 * C111)) +
                                 two * lfma(C011, C201, C110 * C102)) * ri;
    const L C221 = k[2][2][1] - (lfma(C200, C021, lfma(C020, C201, four * C110 * C111)) +
                                 two * lfma(C101, C120, C011 * C210)) * ri;
    const L m4sum = lfma(C011, k[2][1][1], lfma(C101, k[1][2][1], C110 * k[1][1][2]));
    const L m3sum = lfma(C120, C102, lfma(C210, C012, C201 * C021));
    const L C222 = k[2][2][2] -
                   (lfma(four * C111, C111, lfma(C200, k[0][2][2], lfma(C020, k[2][0][2], C002 * k[2][2][0]))) +
                    lfma(four, m4sum, two * m3sum)) * ri +
                   lfma((L)16.0f * C110, C101 * C011,
                        lfma(four, lfma(C101 * C101, C020, lfma(C011 * C011, C200, C110 * C110 * C002)),
                             two * C200 * C020 * C002)) * ri * ri;
    // rates: omega_2 = 1, G2017 eq. 14-16 with o = omega_1
    const L o = om;
    const L w3 = (L)8.0f * (o - two) * lfma((L)3.0f, o, (L)-1.0f - (L)5.0f * o) *
                 rcp(lfma((L)8.0f * lfma((L)-2.0f, o, (L)5.0f), o, lfma(o, lfma((L)9.0f, o, (L)-26.0f), (L)8.0f)));
    const L w4 = (L)8.0f * (o - two) * lfma((L)3.0f, o, o - (L)7.0f) *
                 rcp(lfma(o, lfma((L)8.0f, o, (L)-42.0f), (L)56.0f) - (L)8.0f * o);
    const L w5 = (L)24.0f * (o - two) *
                 lfma((L)4.0f * o, o, lfma(o, lfma((L)-13.0f, o, (L)18.0f), lfma(o, lfma((L)6.0f, o, (L)-11.0f), two))) *
                 rcp((L)16.0f * o * o * (o - (L)6.0f) - two * o * lfma((L)5.0f * o, lfma((L)9.0f, o, (L)-46.0f), (L)216.0f) +
                     lfma(o * lfma((L)3.0f, o, (L)-10.0f), lfma((L)15.0f, o, (L)-28.0f), (L)-48.0f));
    const L rl = rho * (L)0.01;  // lambda; a double literal, so FP64 lanes get 0.01 exactly
    auto lim = [&](L w, L c) {
        const L a = labs_(c);
        return lfma(one - w, a * rcp(rl + a), w);
    };
    const L den = (o - one) * lfma((L)3.0f, o, two - (L)8.0f * o);
    const L rden = rcp(den);
    const L A4 = lfma((L)4.0f * o, o, lfma(two * o, o - (L)6.0f, lfma(o, lfma((L)-3.0f, o, (L)10.0f), (L)-4.0f))) * rden;
    const L B4 = (lfma((L)4.0f * o, lfma((L)9.0f, o, (L)-16.0f), (L)-4.0f * o * o) -
                  two * lfma((L)9.0f * o, o - two, two)) * rden * third;
    // second order (G2015 eq. 55-65)
    const L h = half * ri;
    const L d20 = C200 - C020, d02 = C200 - C002;
    const L Dxu = -h * lfma(o, d20 + d02, C200 + C020 + C002 - K000);
    const L t3oh = (L)3.0f * o * h;
    const L Dyv = lfma(t3oh, d20, Dxu), Dzw = lfma(t3oh, d02, Dxu);
    const L m3o = (L)-3.0f * o * ri;
    const L DxvDyu = m3o * C110, DxwDzu = m3o * C101, DywDzv = m3o * C011;
    const L o1 = one - o;
    const L a3 = rho * lfma((L)-1.5f, o, (L)3.0f);  // 3 rho (1 - o/2)
    const L xD = ux * ux * Dxu, yD = uy * uy * Dyv, zD = uz * uz * Dzw;
    const L E61 = lfma(o1, d20, a3 * (yD - xD));
    const L E64 = lfma(o1, d02, a3 * (zD - xD));
    const L E65 = lfma((L)-1.5f * rho, xD + yD + zD, K000);
    const L s200 = (E61 + E64 + E65) * third;
    const L s020 = lfma((L)-2.0f, E61, E64 + E65) * third;
    const L s002 = lfma((L)-2.0f, E64, E61 + E65) * third;
    const L s110 = o1 * C110, s101 = o1 * C101, s011 = o1 * C011;
    // third order (G2017 eq. 37-42)
    const L P1 = (one - lim(w3, C120 + C102)) * (C120 + C102), M1 = (one - lim(w4, C120 - C102)) * (C120 - C102);
    const L P2 = (one - lim(w3, C210 + C012)) * (C210 + C012), M2 = (one - lim(w4, C210 - C012)) * (C210 - C012);
    const L P3 = (one - lim(w3, C201 + C021)) * (C201 + C021), M3 = (one - lim(w4, C201 - C021)) * (C201 - C021);
    const L s120 = half * (P1 + M1), s102 = half * (P1 - M1);
    const L s210 = half * (P2 + M2), s012 = half * (P2 - M2);
    const L s201 = half * (P3 + M3), s021 = half * (P3 - M3);
    const L s111 = (one - lim(w5, C111)) * C111;
    // fourth order (G2017 eq. 43-48 with omega_6..8 = 1); fifth and sixth order relax to zero
    const L vis = rcp(o) - half;
    const L gA = vis * A4 * rho * (L)(2.0 / 3.0), gB = vis * B4 * rho * (L)(-1.0 / 3.0);
    // eq. 43-45 solved for the three cumulants, with eq. 44 driven by Dyv + Dzw - 2 Dxu (its axis
    // image of eq. 43): each C_abc with two 2-indices follows the gradients of those two axes
    const L c220 = -gA * (Dxu + Dyv), c202 = -gA * (Dxu + Dzw), c022 = -gA * (Dyv + Dzw);
    const L c211 = gB * DywDzv, c121 = gB * DxwDzu, c112 = gB * DxvDyu;
    // back to central moments (G2015 eq. 81-87)
    L q[3][3][3];
    q[0][0][0] = K000;
    q[1][0][0] = -K100; q[0][1][0] = -K010; q[0][0][1] = -K001;
    q[1][1][0] = s110; q[1][0][1] = s101; q[0][1][1] = s011;
    q[2][0][0] = s200; q[0][2][0] = s020; q[0][0][2] = s002;
    q[1][2][0] = s120; q[1][0][2] = s102; q[2][1][0] = s210; q[0][1][2] = s012; q[2][0][1] = s201; q[0][2][1] = s021;
    q[1][1][1] = s111;
    q[2][1][1] = c211 + lfma(s200, s011, two * s101 * s110) * ri;
    q[1][2][1] = c121 + lfma(s020, s101, two * s110 * s011) * ri;
    q[1][1][2] = c112 + lfma(s002, s110, two * s011 * s101) * ri;
    q[2][2][0] = c220 + lfma(s020, s200, two * s110 * s110) * ri;
    q[0][2][2] = c022 + lfma(s002, s020, two * s011 * s011) * ri;
    q[2][0][2] = c202 + lfma(s200, s002, two * s101 * s101) * ri;
    q[1][2][2] = (lfma(s020, s102, lfma(s002, s120, four * s011 * s111)) + two * lfma(s110, s012, s101 * s021)) * ri;
    q[2][1][2] = (lfma(s002, s210, lfma(s200, s012, four * s101 * s111)) + two * lfma(s011, s201, s110 * s102)) * ri;
    q[2][2][1] = (lfma(s200, s021, lfma(s020, s201, four * s110 * s111)) + two * lfma(s101, s120, s011 * s210)) * ri;
    const L n4sum = lfma(s011, q[2][1][1], lfma(s101, q[1][2][1], s110 * q[1][1][2]));
    const L n3sum = lfma(s120, s102, lfma(s210, s012, s201 * s021));
    q[2][2][2] = (lfma(four * s111, s111, lfma(s200, q[0][2][2], lfma(s020, q[2][0][2], s002 * q[2][2][0]))) +
                  lfma(four, n4sum, two * n3sum)) * ri -
                 lfma((L)16.0f * s110, s101 * s011,
                      lfma(four, lfma(s101 * s101, s020, lfma(s011 * s011, s200, s110 * s110 * s002)),
                           two * s200 * s020 * s002)) * ri * ri;
    // backward transform: x pass, y pass, z pass (G2015 eq. 88-96)
    const Axis<L> ax = make_axis(ux, ux * ux), ay = make_axis(uy, uy * uy), az = make_axis(uz, uz * uz);
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            L m, z, p;
            tri(q[0][b][c], q[1][b][c], q[2][b][c], ax, m, z, p);
            q[0][b][c] = m; q[1][b][c] = z; q[2][b][c] = p;
        }
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            L m, z, p;
            tri(q[a][0][c], q[a][1][c], q[a][2][c], ay, m, z, p);
            q[a][0][c] = m; q[a][1][c] = z; q[a][2][c] = p;
        }
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) {
            L m, z, p;
            tri(q[a][b][0], q[a][b][1], q[a][b][2], az, m, z, p);
            f[vid(a - 1, b - 1, -1)] = m;
            f[vid(a - 1, b - 1, 0)] = z;
            f[vid(a - 1, b - 1, 1)] = p;
        }
}

}  // namespace lbm
