// lbm_device.cuh - device code of the fused D3Q27 collide-and-stream step (sm_103a).
//
// One thread per cell, x fastest (a warp covers 32 consecutive x of one row), SoA populations
// A[v][z][y][x].  Streaming is the AA pattern: on an even step a cell reads its own slots A[x][v]
// and writes post-collision f*_v into A[x][opp v]; on an odd step it reads A[x-c_v][opp v] and
// writes f*_v into A[x+c_v][v].  Every slot a thread reads is written only by that thread, so
// one array serves in place with no race.  Boundaries are folded into the gather by the cell
// class byte:
//   half-way bounce-back from a solid neighbour x-c_v   (BounceBackWallHalf.h:114-125)
//       even step reads A[x-c_v][opp v], odd step reads A[x][v]  (the swapped slot);
//   moving-wall nodes (flag -1, InletVelocityMovingWall.h:31-55) keep their own 27-value state in
//       a 3-level side table; neighbours stream their state of one step earlier (StreamingAB.h:62-65);
//   equilibrium velocity-inlet nodes (InletVelocityEquilibrium.h:115-167) are not updated: their
//       neighbours rebuild f_eq(u_b, rho_b) from the moments that the two interior "probe" cells
//       stored two steps earlier (3-level table);
//   density-interpolated outlets (OutletDensityInterpolated.h:170-252) read the upstream cell's and
//       their own post-collision values of the previous step from a 2-parity side table.
// Periodicity is by index wrap.  The same gather serves the read-only kernels (moments, diagnostics).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

namespace lbm {

#define LBM_HD __host__ __device__ __forceinline__
#define LBM_D __device__ __forceinline__

// ---- cell class byte ---------------------------------------------------------------------------
enum : uint8_t { CLS_SOLID = 0, CLS_BULK = 1, CLS_EDGE = 2, CLS_LID = 3, CLS_INLET = 4, CLS_OUTLET = 5 };
enum : uint8_t {
    BIT_PROBE1 = 1u << 3,   // interior neighbour 1 of an equilibrium inlet: stores rho, ux
    BIT_PROBE2 = 1u << 4,   // interior neighbour 2: stores ux
    BIT_OUTUP = 1u << 5,    // upstream neighbour of an outlet: stores its incoming-direction f*
    BIT_REFBULK = 1u << 6,  // reference flag == 1 (cells the error monitor sums over)
};
constexpr uint8_t CLS_MASK = 7;

// ---- D3Q27 in the reference's order (models/D3Q27/D3Q27.h:81-124) ------------------------------
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
LBM_HD constexpr double wgt(int v) {
    return (cx(v) * cx(v) + cy(v) * cy(v) + cz(v) * cz(v)) == 0   ? 8.0 / 27.0
           : (cx(v) * cx(v) + cy(v) * cy(v) + cz(v) * cz(v)) == 1 ? 2.0 / 27.0
           : (cx(v) * cx(v) + cy(v) * cy(v) + cz(v) * cz(v)) == 2 ? 1.0 / 54.0
                                                                   : 1.0 / 216.0;
}
// the 9 directions with c_x = -s (s = +1: outlet facing +x) as used by the outlet side table
LBM_HD constexpr int outlet_dir(int s, int k) {
    constexpr int neg[9] = {2, 8, 10, 11, 15, 19, 21, 24, 25};  // c_x = -1
    constexpr int pos[9] = {1, 7, 9, 12, 16, 20, 22, 23, 26};   // c_x = +1
    return s > 0 ? neg[k] : pos[k];
}
LBM_HD constexpr int outlet_slot(int v) {  // k with outlet_dir(+-1, k) == v
    constexpr int t[27] = {-1, 0, 0, -1, -1, -1, -1, 1, 1, 2, 2, 3, 3, -1, -1, 4, 4, -1, -1, 5, 5, 6, 6, 7, 7, 8, 8};
    return t[v];
}

template <int I, int N, class F>
LBM_D void sfor(F&& f) {
    if constexpr (I < N) {
        f(std::integral_constant<int, I>{});
        sfor<I + 1, N>(f);
    }
}

// ---- storage types -------------------------------------------------------------------------------
struct StF64 { using T = double; using R = double; static constexpr int kind = 0; };
struct StF32 { using T = float;  using R = float;  static constexpr int kind = 1; };
struct StF16 { using T = __half; using R = float;  static constexpr int kind = 2; };

// kernel parameters (identical for all storage types; pointers are typed inside the kernels)
struct Params {
    void* f;                 // populations, 27*N of S::T
    const uint8_t* cls;      // class byte per cell
    const int32_t* aux;      // side-table index per cell (special nodes and their helpers)
    int nx, ny, nz;
    int wrap[3];
    long long N;
    int m;                   // index of the state being consumed (steps done so far)
    double tau, cles18, nu;  // relaxation time, 18*CLES, lattice viscosity (inlet rho_b)
    double F[3];             // body force
    float rho0, scale, inv_scale;  // FP16-deviation encoding
    // moving-wall nodes
    void* lid_state;         // [3][27][n_lid] of S::R
    const float* lid_n;      // [3][n_lid] outward normals
    const float* lid_u;      // [3][n_lid] wall velocities
    int n_lid;
    // equilibrium inlets
    void* in_probe;          // [3][3][n_in] of S::R : rho1, ux1, ux2 per level
    const float* in_u;       // [3][n_in]
    const int32_t* in_dir;   // +1: normal +x (interior at -x), -1: normal -x
    int n_in;
    // density-interpolated outlets
    void* out_save;          // [2][2][9][n_out] of S::R : parity, {upstream, own}, k, node
    const float* out_rho;    // prescribed density
    const int32_t* out_dir;  // +1: normal +x, -1: normal -x
    int n_out;
    // per-step options
    double* acc;             // time-average accumulators [10][N] (nullptr: off)
};

template <class S>
struct Codec;
template <>
struct Codec<StF64> {
    LBM_D static double dec(const double* A, long long i, double, const Params&) { return A[i]; }
    LBM_D static void enc(double* A, long long i, double v, double, const Params&) { A[i] = v; }
};
template <>
struct Codec<StF32> {
    LBM_D static float dec(const float* A, long long i, float, const Params&) { return __ldg(A + i); }
    LBM_D static void enc(float* A, long long i, float v, float, const Params&) { A[i] = v; }
};
template <>
struct Codec<StF16> {
    // f = w_v rho0 + h 2^-s, stored h = (f - w_v rho0) 2^s  (the FP16-deviation encoding)
    LBM_D static float dec(const __half* A, long long i, float wr, const Params& p) {
        return fmaf(__half2float(A[i]), p.inv_scale, wr);
    }
    LBM_D static void enc(__half* A, long long i, float v, float wr, const Params& p) {
        A[i] = __float2half_rn((v - wr) * p.scale);
    }
};

// ---- equilibrium (second-order polynomial of the reference, e.g. OmegaLES.h:275-294) ----------
template <int V, class R>
LBM_D R feq(R r, R ux, R uy, R uz, R u2) {
    const R cu = (R)cx(V) * ux + (R)cy(V) * uy + (R)cz(V) * uz;
    return (R)wgt(V) * r * ((R)1 + (R)3 * cu + (R)4.5 * cu * cu - (R)1.5 * u2);
}

// ---- cell geometry: wrapped neighbour coordinates -----------------------------------------------
struct Cell {
    int x, y, z;
    long long idx;
    int X[3];         // x-1, x, x+1 (wrapped)
    long long Y[3];   // (y-1, y, y+1) * nx (wrapped)
    long long Z[3];   // (z-1, z, z+1) * nx*ny (wrapped)
    unsigned oob;     // bit (2*axis + (d>0)): the neighbour at d on that axis leaves a non-periodic box
};
LBM_D void make_cell(const Params& p, int x, int y, int z, Cell& c) {
    c.x = x; c.y = y; c.z = z;
    const long long sxy = (long long)p.nx * p.ny;
    c.idx = x + (long long)p.nx * y + sxy * z;
    c.X[0] = x == 0 ? p.nx - 1 : x - 1; c.X[1] = x; c.X[2] = x == p.nx - 1 ? 0 : x + 1;
    c.Y[0] = (long long)(y == 0 ? p.ny - 1 : y - 1) * p.nx; c.Y[1] = (long long)y * p.nx;
    c.Y[2] = (long long)(y == p.ny - 1 ? 0 : y + 1) * p.nx;
    c.Z[0] = (long long)(z == 0 ? p.nz - 1 : z - 1) * sxy; c.Z[1] = (long long)z * sxy;
    c.Z[2] = (long long)(z == p.nz - 1 ? 0 : z + 1) * sxy;
    c.oob = 0;
    if (!p.wrap[0]) c.oob |= (x == 0 ? 1u : 0u) | (x == p.nx - 1 ? 2u : 0u);
    if (!p.wrap[1]) c.oob |= (y == 0 ? 4u : 0u) | (y == p.ny - 1 ? 8u : 0u);
    if (!p.wrap[2]) c.oob |= (z == 0 ? 16u : 0u) | (z == p.nz - 1 ? 32u : 0u);
}
// index of the cell at offset (dx,dy,dz) in {-1,0,1}^3
template <int DX, int DY, int DZ>
LBM_D long long nbr(const Cell& c) { return c.X[DX + 1] + c.Y[DY + 1] + c.Z[DZ + 1]; }
template <int DX, int DY, int DZ>
LBM_D bool nbr_oob(const Cell& c) {
    unsigned m = 0;
    if (DX < 0) m |= 1u; if (DX > 0) m |= 2u;
    if (DY < 0) m |= 4u; if (DY > 0) m |= 8u;
    if (DZ < 0) m |= 16u; if (DZ > 0) m |= 32u;
    return (c.oob & m) != 0;
}

// level of a 3-level side table for step index k (k may be -1 or -2)
LBM_D int lvl3(int k) { return ((k % 3) + 3) % 3; }

template <class S>
LBM_D typename S::R wr_of(int v, const Params& p) {
    if constexpr (S::kind == 2) return (float)wgt(v) * p.rho0; else return (typename S::R)0;
}

// ---- gather: the pre-collision populations df_m(x, .) of a non-solid, non-inlet cell ----------
// DRAG: accumulate the momentum-exchange force over solid links (read-only kernels only).
template <class S, bool ODD, bool DRAG>
LBM_D void gather(const Params& p, const Cell& c, int cl, typename S::R (&f)[27], typename S::R (&drag)[3]) {
    using R = typename S::R;
    using T = typename S::T;
    const T* A = (const T*)p.f;
    const long long N = p.N;
    if (cl == CLS_LID) {
        const R* st = (const R*)p.lid_state + (long long)lvl3(p.m) * 27 * p.n_lid;
        const int id = p.aux[c.idx];
        sfor<0, 27>([&](auto vc) { constexpr int V = decltype(vc)::value; f[V] = st[V * p.n_lid + id]; });
        return;
    }
    if (cl == CLS_BULK || p.m == 0) {
        // plain AA read; at m = 0 every cell reads its own (initial) slots
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            const R wr = wr_of<S>(V, p);
            if (ODD) f[V] = Codec<S>::dec(A, opp(V) * N + nbr<-cx(V), -cy(V), -cz(V)>(c), wr, p);
            else     f[V] = Codec<S>::dec(A, V * N + c.idx, wr, p);
        });
        return;
    }
    // EDGE or OUTLET, m >= 1: per-link rules
    const int osgn = (cl == CLS_OUTLET) ? p.out_dir[p.aux[c.idx]] : 0;
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        const R wr = wr_of<S>(V, p);
        if (osgn != 0 && cx(V) == -osgn) { f[V] = (R)0; return; }  // interpolated below
        if (V == 0 || nbr_oob<-cx(V), -cy(V), -cz(V)>(c)) {
            // rest population, or a link leaving the box (rejected at set-up): own/plain read
            if (ODD) f[V] = V == 0 ? Codec<S>::dec(A, c.idx, wr, p) : (R)0;
            else     f[V] = Codec<S>::dec(A, V * N + c.idx, wr, p);
            return;
        }
        const long long nb = nbr<-cx(V), -cy(V), -cz(V)>(c);
        const int ncl = p.cls[nb] & CLS_MASK;
        if (ncl == CLS_SOLID) {
            // half-way bounce-back: f_v(x) = f*_{opp v}(x) of the previous step
            R b = ODD ? Codec<S>::dec(A, V * N + c.idx, wr, p) : Codec<S>::dec(A, opp(V) * N + nb, wr, p);
            f[V] = b;
            if (DRAG) {  // fluid momentum lost through the link: b*c_{opp v} - b*c_v = -2 b c_v
                drag[0] -= (R)(2 * cx(V)) * b; drag[1] -= (R)(2 * cy(V)) * b; drag[2] -= (R)(2 * cz(V)) * b;
            }
        } else if (ncl == CLS_LID) {
            const R* st = (const R*)p.lid_state + (long long)lvl3(p.m - 1) * 27 * p.n_lid;
            f[V] = st[V * p.n_lid + p.aux[nb]];
        } else if (ncl == CLS_INLET) {
            const int id = p.aux[nb];
            const R* pr = (const R*)p.in_probe + (long long)lvl3(p.m - 2) * 3 * p.n_in;
            const R r1 = pr[id], ux1 = pr[p.n_in + id], ux2 = pr[2 * p.n_in + id];
            const R ub0 = p.in_u[id], ub1 = p.in_u[p.n_in + id], ub2 = p.in_u[2 * p.n_in + id];
            R rb;
            if (p.in_dir[id] > 0) rb = r1 + (R)p.nu / (R)3 * ((ux1 - ux2) - (ub0 - ux1));
            else                  rb = r1 + (R)p.nu / (R)3 * ((ux1 - ub0) - (ux2 - ux1));
            f[V] = feq<V>(rb, ub0, ub1, ub2, ub0 * ub0 + ub1 * ub1 + ub2 * ub2);
        } else {
            if (ODD) f[V] = Codec<S>::dec(A, opp(V) * N + nb, wr, p);
            else     f[V] = Codec<S>::dec(A, V * N + c.idx, wr, p);
        }
    });
    if (osgn != 0) {
        // OutletDensityInterpolated.h:200-221: incoming = cs f*(x-n) + (1-cs) f*(x); then
        // f += f_eq(u, 1) - f_eq(u, rho) with u from the prescribed density
        const int id = p.aux[c.idx];
        const R* sv = (const R*)p.out_save + (long long)((p.m - 1) & 1) * 18 * p.n_out;
        const R cs = (R)0.57735026918962576451;  // 1/sqrt(3), LBMConstants.h:103
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            if constexpr (cx(V) != 0) {
                if (cx(V) == -osgn) {
                    const int k = outlet_slot(V);
                    f[V] = cs * sv[k * p.n_out + id] + ((R)1 - cs) * sv[(9 + k) * p.n_out + id];
                }
            }
        });
        R r = 0, jx = 0, jy = 0, jz = 0;
        sfor<0, 27>([&](auto vc) { constexpr int V = decltype(vc)::value; r += f[V]; });
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            if (cx(V)) jx += (R)cx(V) * f[V];
            if (cy(V)) jy += (R)cy(V) * f[V];
            if (cz(V)) jz += (R)cz(V) * f[V];
        });
        const R dens = (R)p.out_rho[id];
        const R ux = jx / dens, uy = jy / dens, uz = jz / dens, u2 = ux * ux + uy * uy + uz * uz;
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            f[V] = f[V] - feq<V>(r, ux, uy, uz, u2) + feq<V>((R)1, ux, uy, uz, u2);
        });
    }
}

// state df_m of an equilibrium-inlet node: f_eq(u_b, rho_b) with rho_b from the probe moments of
// step m-1 (InletVelocityEquilibrium.h:148-160 run at the end of step m-1)
template <class S>
LBM_D void inlet_state(const Params& p, const Cell& c, typename S::R (&f)[27]) {
    using R = typename S::R;
    const int id = p.aux[c.idx];
    const R* pr = (const R*)p.in_probe + (long long)lvl3(p.m - 1) * 3 * p.n_in;
    const R r1 = pr[id], ux1 = pr[p.n_in + id], ux2 = pr[2 * p.n_in + id];
    const R ub0 = p.in_u[id], ub1 = p.in_u[p.n_in + id], ub2 = p.in_u[2 * p.n_in + id];
    R rb;
    if (p.in_dir[id] > 0) rb = r1 + (R)p.nu / (R)3 * ((ux1 - ux2) - (ub0 - ux1));
    else                  rb = r1 + (R)p.nu / (R)3 * ((ux1 - ub0) - (ux2 - ux1));
    const R u2 = ub0 * ub0 + ub1 * ub1 + ub2 * ub2;
    sfor<0, 27>([&](auto vc) { constexpr int V = decltype(vc)::value; f[V] = feq<V>(rb, ub0, ub1, ub2, u2); });
}

// ---- moments in the reference's summation order (MomentDensityVelocityN27.h:212-228) ----------
template <class R>
LBM_D void moments(const R (&f)[27], const Params& p, R& rho, R& jx, R& jy, R& jz, R& ux, R& uy, R& uz) {
    rho = 0; jx = 0; jy = 0; jz = 0;
    sfor<0, 27>([&](auto vc) { constexpr int V = decltype(vc)::value; rho += f[V]; });
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        if (cx(V)) jx += (R)cx(V) * f[V];
        if (cy(V)) jy += (R)cy(V) * f[V];
        if (cz(V)) jz += (R)cz(V) * f[V];
    });
    const R ri = (R)1 / rho;
    ux = (jx + (R)0.5 * (R)p.F[0]) * ri;
    uy = (jy + (R)0.5 * (R)p.F[1]) * ri;
    uz = (jz + (R)0.5 * (R)p.F[2]) * ri;
}

// ---- raw second moments via z-, y-, x-pair sums ----------------------------------------------------
template <class R>
LBM_D void second_moments(const R (&f)[27], R& Mxx, R& Myy, R& Mzz, R& Mxy, R& Mxz, R& Myz) {
    R xx = 0, yy = 0, zz = 0, xy = 0, xz = 0, yz = 0;
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        if (cx(V)) xx += f[V];
        if (cy(V)) yy += f[V];
        if (cz(V)) zz += f[V];
        if (cx(V) * cy(V)) xy += (R)(cx(V) * cy(V)) * f[V];
        if (cx(V) * cz(V)) xz += (R)(cx(V) * cz(V)) * f[V];
        if (cy(V) * cz(V)) yz += (R)(cy(V) * cz(V)) * f[V];
    });
    Mxx = xx; Myy = yy; Mzz = zz; Mxy = xy; Mxz = xz; Myz = yz;
}

// ---- relaxation rate ----------------------------------------------------------------------------
// Smagorinsky (OmegaLES.h:312-357): Pi = sum c c (f - f_eq) = M - rho (u u + I/3),
// tau_LES = tau/2 + sqrt(tau^2 + 18 CLES |Pi| / rho)/2
template <class R, int CLOS>
LBM_D R relax_rate(const Params& p, R rho, R ux, R uy, R uz, R Mxx, R Myy, R Mzz, R Mxy, R Mxz, R Myz) {
    const R tau = (R)p.tau;
    if constexpr (CLOS == 0) {
        return (R)1 / tau;
    } else {
        const R third = rho * ((R)1 / (R)3);
        const R pxx = Mxx - rho * ux * ux - third, pyy = Myy - rho * uy * uy - third, pzz = Mzz - rho * uz * uz - third;
        const R pxy = Mxy - rho * ux * uy, pxz = Mxz - rho * ux * uz, pyz = Myz - rho * uy * uz;
        const R PI2 = pxx * pxx + pyy * pyy + pzz * pzz + (R)2 * (pxy * pxy + pxz * pxz + pyz * pyz);
        const R PI = sqrt(PI2);
        const R tles = tau * (R)0.5 + (R)0.5 * sqrt(tau * tau + (R)p.cles18 / rho * PI);
        return (R)1 / tles;
    }
}

// ---- SRT (CollisionSRTTurbulent.h:386-391), Guo forcing when F != 0 --------------------------------
template <class R>
LBM_D void collide_srt(R (&f)[27], const Params& p, R rho, R ux, R uy, R uz, R om, bool force) {
    const R u2 = ux * ux + uy * uy + uz * uz;
    const R gf = (R)1 - (R)0.5 * om;
    const R Fx = (R)p.F[0], Fy = (R)p.F[1], Fz = (R)p.F[2];
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        R out = f[V] - (f[V] - feq<V>(rho, ux, uy, uz, u2)) * om;
        if (force) {
            const R cu = (R)cx(V) * ux + (R)cy(V) * uy + (R)cz(V) * uz;
            const R s = ((R)3 * ((R)cx(V) - ux) + (R)9 * cu * (R)cx(V)) * Fx +
                        ((R)3 * ((R)cy(V) - uy) + (R)9 * cu * (R)cy(V)) * Fy +
                        ((R)3 * ((R)cz(V) - uz) + (R)9 * cu * (R)cz(V)) * Fz;
            out += gf * (R)wgt(V) * s;
        }
        f[V] = out;
    });
}

// ---- cumulant collision, Geier 2015 with omega_2..omega_10 = 1 -----------------------------------
// Same operator as CollisionCumD3Q27Turbulent2015.h:80-485, written in closed form: with all higher
// relaxation rates equal to one, every post-collision cumulant above second order is zero, so only
// the second-order central moments are needed from the forward transform and the backward
// (chimera, G2015 eq. 88-96) transform takes the products of eq. 81-84.
template <class R>
LBM_D void tri_bwd(R k0, R k1, R k2, R u, R A, R B, R onemu2, R& m, R& z, R& p) {
    // (k0,k1,k2) central moments along one axis -> populations (m, 0, p) of that axis
    m = k0 * A + k1 * B + (R)0.5 * k2;   // 0.5 (k0 (u^2-u) + k1 (2u-1) + k2)
    p = m + k0 * u + k1;                  // 0.5 (k0 (u^2+u) + k1 (2u+1) + k2)
    z = k0 * onemu2 - (R)2 * u * k1 - k2;
}

template <class R>
LBM_D void collide_cum15(R (&f)[27], R rho, R jx, R jy, R jz, R ux, R uy, R uz, R om,
                         R Mxx, R Myy, R Mzz, R Mxy, R Mxz, R Myz) {
    const R ri = (R)1 / rho;
    // central moments (k_100 = j_x - rho u_x carries the half-force shift, G2015 eq. 85-87)
    const R k100 = jx - rho * ux, k010 = jy - rho * uy, k001 = jz - rho * uz;
    const R C200 = Mxx + ux * (rho * ux - (R)2 * jx);
    const R C020 = Myy + uy * (rho * uy - (R)2 * jy);
    const R C002 = Mzz + uz * (rho * uz - (R)2 * jz);
    const R C110 = Mxy - ux * jy - uy * jx + rho * ux * uy;
    const R C101 = Mxz - ux * jz - uz * jx + rho * ux * uz;
    const R C011 = Myz - uy * jz - uz * jy + rho * uy * uz;
    // relaxation, G2015 eq. 55-63 with omega_2 = 1
    const R h = (R)0.5 * ri;
    const R Dxu = -om * h * ((R)2 * C200 - C020 - C002) - h * (C200 + C020 + C002 - rho);
    const R Dyv = Dxu + (R)3 * om * h * (C200 - C020);
    const R Dzw = Dxu + (R)3 * om * h * (C200 - C002);
    const R o1 = (R)1 - om;
    const R a = (R)3 * rho * ((R)1 - om * (R)0.5);
    const R xD = ux * ux * Dxu, yD = uy * uy * Dyv, zD = uz * uz * Dzw;
    const R E61 = o1 * (C200 - C020) - a * (xD - yD);
    const R E64 = o1 * (C200 - C002) - a * (xD - zD);
    const R E65 = rho - (R)1.5 * rho * (xD + yD + zD);
    const R t3 = (R)1 / (R)3;
    const R s200 = t3 * (E61 + E64 + E65);
    const R s020 = t3 * (E64 - (R)2 * E61 + E65);
    const R s002 = t3 * (E61 - (R)2 * E64 + E65);
    const R s110 = o1 * C110, s101 = o1 * C101, s011 = o1 * C011;
    // post-collision central moments from cumulants (G2015 eq. 81-84; third order and the
    // relaxed higher cumulants are zero)
    const R q211 = (s200 * s011 + (R)2 * s101 * s110) * ri;
    const R q121 = (s020 * s101 + (R)2 * s110 * s011) * ri;
    const R q112 = (s002 * s110 + (R)2 * s011 * s101) * ri;
    const R q220 = (s020 * s200 + (R)2 * s110 * s110) * ri;
    const R q022 = (s002 * s020 + (R)2 * s011 * s011) * ri;
    const R q202 = (s200 * s002 + (R)2 * s101 * s101) * ri;
    const R q222 = (s200 * q022 + s020 * q202 + s002 * q220 + (R)4 * (s011 * q211 + s101 * q121 + s110 * q112)) * ri -
                   ((R)16 * s110 * s101 * s011 +
                    (R)4 * (s101 * s101 * s020 + s011 * s011 * s200 + s110 * s110 * s002) +
                    (R)2 * s200 * s020 * s002) * ri * ri;
    const R q100 = -k100, q010 = -k010, q001 = -k001;
    // backward chimera transform: x pass (9 triplets over (oy, oz)), then y, then z
    const R Ax = (R)0.5 * (ux * ux - ux), Bx = ux - (R)0.5, Cx = (R)1 - ux * ux;
    const R Ay = (R)0.5 * (uy * uy - uy), By = uy - (R)0.5, Cy = (R)1 - uy * uy;
    const R Az = (R)0.5 * (uz * uz - uz), Bz = uz - (R)0.5, Cz = (R)1 - uz * uz;
    R g[3][3][3];  // [sx][oy][oz]
    const R zero = (R)0;
    tri_bwd(rho,  q100, s200, ux, Ax, Bx, Cx, g[0][0][0], g[1][0][0], g[2][0][0]);
    tri_bwd(q001, s101, zero, ux, Ax, Bx, Cx, g[0][0][1], g[1][0][1], g[2][0][1]);
    tri_bwd(s002, zero, q202, ux, Ax, Bx, Cx, g[0][0][2], g[1][0][2], g[2][0][2]);
    tri_bwd(q010, s110, zero, ux, Ax, Bx, Cx, g[0][1][0], g[1][1][0], g[2][1][0]);
    tri_bwd(s011, zero, q211, ux, Ax, Bx, Cx, g[0][1][1], g[1][1][1], g[2][1][1]);
    tri_bwd(zero, q112, zero, ux, Ax, Bx, Cx, g[0][1][2], g[1][1][2], g[2][1][2]);
    tri_bwd(s020, zero, q220, ux, Ax, Bx, Cx, g[0][2][0], g[1][2][0], g[2][2][0]);
    tri_bwd(zero, q121, zero, ux, Ax, Bx, Cx, g[0][2][1], g[1][2][1], g[2][2][1]);
    tri_bwd(q022, zero, q222, ux, Ax, Bx, Cx, g[0][2][2], g[1][2][2], g[2][2][2]);
    R hh[3][3][3];  // [sx][sy][oz]
#pragma unroll
    for (int sx = 0; sx < 3; sx++)
#pragma unroll
        for (int oz = 0; oz < 3; oz++)
            tri_bwd(g[sx][0][oz], g[sx][1][oz], g[sx][2][oz], uy, Ay, By, Cy, hh[sx][0][oz], hh[sx][1][oz], hh[sx][2][oz]);
    R o[3][3][3];  // [sx][sy][sz]
#pragma unroll
    for (int sx = 0; sx < 3; sx++)
#pragma unroll
        for (int sy = 0; sy < 3; sy++)
            tri_bwd(hh[sx][sy][0], hh[sx][sy][1], hh[sx][sy][2], uz, Az, Bz, Cz, o[sx][sy][0], o[sx][sy][1], o[sx][sy][2]);
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        f[V] = o[cx(V) + 1][cy(V) + 1][cz(V) + 1];
    });
}

// ---- the fused step kernel ----------------------------------------------------------------------------
// COLL: 0 SRT, 1 cumulant-2015.  CLOS: 0 none, 1 Smagorinsky.
template <class S, int COLL, int CLOS, bool ODD>
__global__ void __launch_bounds__(128) k_step(Params p) {
    using R = typename S::R;
    using T = typename S::T;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= p.nx) return;
    Cell c;
    make_cell(p, x, blockIdx.y, blockIdx.z, c);
    const uint8_t fl = p.cls[c.idx];
    const int cl = fl & CLS_MASK;
    if (cl == CLS_SOLID) return;
    R f[27];
    if (cl == CLS_INLET) {
        // node is not updated; only the time average (MomentTimeAvg runs over every cell) needs it
        if (p.acc) {
            inlet_state<S>(p, c, f);
            R rho, jx, jy, jz, ux, uy, uz;
            moments(f, p, rho, jx, jy, jz, ux, uy, uz);
            double* a = p.acc;
            const long long N = p.N;
            a[c.idx] += rho; a[N + c.idx] += ux; a[2 * N + c.idx] += uy; a[3 * N + c.idx] += uz;
            a[4 * N + c.idx] += (double)ux * ux; a[5 * N + c.idx] += (double)uy * uy; a[6 * N + c.idx] += (double)uz * uz;
            a[7 * N + c.idx] += (double)ux * uy; a[8 * N + c.idx] += (double)ux * uz; a[9 * N + c.idx] += (double)uy * uz;
        }
        return;
    }
    R drag[3] = {0, 0, 0};
    gather<S, ODD, false>(p, c, cl, f, drag);

    R rho, jx, jy, jz, ux, uy, uz;
    moments(f, p, rho, jx, jy, jz, ux, uy, uz);
    if (fl & (BIT_PROBE1 | BIT_PROBE2)) {
        R* pr = (R*)p.in_probe + (long long)lvl3(p.m) * 3 * p.n_in;
        const int id = p.aux[c.idx];
        if (fl & BIT_PROBE1) { pr[id] = rho; pr[p.n_in + id] = ux; }
        else pr[2 * p.n_in + id] = ux;
    }
    if (p.acc) {
        double* a = p.acc;
        const long long N = p.N;
        a[c.idx] += rho; a[N + c.idx] += ux; a[2 * N + c.idx] += uy; a[3 * N + c.idx] += uz;
        a[4 * N + c.idx] += (double)ux * ux; a[5 * N + c.idx] += (double)uy * uy; a[6 * N + c.idx] += (double)uz * uz;
        a[7 * N + c.idx] += (double)ux * uy; a[8 * N + c.idx] += (double)ux * uz; a[9 * N + c.idx] += (double)uy * uz;
    }
    R Mxx, Myy, Mzz, Mxy, Mxz, Myz;
    second_moments(f, Mxx, Myy, Mzz, Mxy, Mxz, Myz);
    const R om = relax_rate<R, CLOS>(p, rho, ux, uy, uz, Mxx, Myy, Mzz, Mxy, Mxz, Myz);
    const bool force = p.F[0] != 0.0 || p.F[1] != 0.0 || p.F[2] != 0.0;
    if constexpr (COLL == 0) collide_srt(f, p, rho, ux, uy, uz, om, force);
    else collide_cum15(f, rho, jx, jy, jz, ux, uy, uz, om, Mxx, Myy, Mzz, Mxy, Mxz, Myz);

    if (cl == CLS_LID) {
        // InletVelocityMovingWall.h:40-53: for n.c_v > 0, df(x, opp v) = f*_v - 6 w_v rho (c_v . u_w);
        // the other components keep their value.  Written to the next level.
        const int id = p.aux[c.idx];
        const int nl = p.n_lid;
        const R* cur = (const R*)p.lid_state + (long long)lvl3(p.m) * 27 * nl;
        R* nxt = (R*)p.lid_state + (long long)lvl3(p.m + 1) * 27 * nl;
        const R n0 = p.lid_n[id], n1 = p.lid_n[nl + id], n2 = p.lid_n[2 * nl + id];
        const R w0 = p.lid_u[id], w1 = p.lid_u[nl + id], w2 = p.lid_u[2 * nl + id];
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            constexpr int O = opp(V);
            // component O is set from f*_V when n.c_V > 0, else it keeps its value
            if (n0 * (R)cx(V) + n1 * (R)cy(V) + n2 * (R)cz(V) > (R)0)
                nxt[O * nl + id] = f[V] - (R)6 * (R)wgt(V) * rho * ((R)cx(V) * w0 + (R)cy(V) * w1 + (R)cz(V) * w2);
            else
                nxt[O * nl + id] = cur[O * nl + id];
        });
        return;
    }
    if (fl & BIT_OUTUP) {
        const int id = p.aux[c.idx];
        const int s = p.out_dir[id];
        R* sv = (R*)p.out_save + (long long)(p.m & 1) * 18 * p.n_out;
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            if constexpr (cx(V) != 0) if (cx(V) == -s) sv[outlet_slot(V) * p.n_out + id] = f[V];
        });
    }
    if (cl == CLS_OUTLET) {
        const int id = p.aux[c.idx];
        const int s = p.out_dir[id];
        R* sv = (R*)p.out_save + (long long)(p.m & 1) * 18 * p.n_out;
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            if constexpr (cx(V) != 0) if (cx(V) == -s) sv[(9 + outlet_slot(V)) * p.n_out + id] = f[V];
        });
    }
    // scatter (AA)
    T* A = (T*)p.f;
    const long long N = p.N;
    if (cl == CLS_BULK) {
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            const R wr = wr_of<S>(V, p);
            if (ODD) Codec<S>::enc(A, V * N + nbr<cx(V), cy(V), cz(V)>(c), f[V], wr, p);
            else     Codec<S>::enc(A, opp(V) * N + c.idx, f[V], wr, p);
        });
    } else {
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            const R wr = wr_of<S>(V, p);
            if (ODD) {
                if (!nbr_oob<cx(V), cy(V), cz(V)>(c)) Codec<S>::enc(A, V * N + nbr<cx(V), cy(V), cz(V)>(c), f[V], wr, p);
            } else {
                Codec<S>::enc(A, opp(V) * N + c.idx, f[V], wr, p);
            }
        });
    }
}

}  // namespace lbm
