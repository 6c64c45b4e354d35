// lbm_device.cuh - device code of the fused D3Q27 collide-and-stream step (sm_103a).
//
// One thread per cell, x fastest (a warp covers 32 consecutive x of one row), SoA populations
// A[v][z][y][x].  Streaming is the AA pattern: on an even step a cell reads its own slots A[x][v]
// and writes post-collision f*_v into A[x][opp v]; on an odd step it reads A[x-c_v][opp v] and
// writes f*_v into A[x+c_v][v].  Every slot a thread reads is written only by that thread, so
// one array serves in place with no race.  Boundaries are folded into the gather by the cell
// class byte:
//   half-way bounce-back from a solid neighbour x-c_v   (BounceBackWallHalf.h:38-49)
//       even step reads A[x-c_v][opp v], odd step reads A[x][v]  (the swapped slot);
//   moving-wall nodes (flag -1, InletVelocityMovingWall.h:31-55) keep their own 27-value state in
//       a 3-level side table; neighbours stream their state of one step earlier (StreamingAB.h:62-65);
//   equilibrium velocity-inlet nodes (InletVelocityEquilibrium.h:51-103) are not updated: their
//       neighbours rebuild f_eq(u_b, rho_b) from the moments that the two interior "probe" cells
//       stored two steps earlier (3-level table);
//   density-interpolated outlets (OutletDensityInterpolated.h:170-252) read the upstream cell's and
//       their own post-collision values of the previous step from a 2-parity side table.
// Periodicity is by index wrap.  Bulk cells away from a periodic seam (almost all cells) take a
// fast path: every access is one precomputed per-direction base address plus the cell index.
// The same general gather serves the read-only kernels (moments, diagnostics, probe).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#define LBM_HD __host__ __device__ __forceinline__
#define LBM_D __device__ __forceinline__

#include "lbm_math.cuh"
#include "lbm_mlp.cuh"

namespace lbm {

// ---- cell class byte ---------------------------------------------------------------------------
enum : uint8_t { CLS_SOLID = 0, CLS_BULK = 1, CLS_EDGE = 2, CLS_LID = 3, CLS_INLET = 4, CLS_OUTLET = 5, CLS_SYM = 6 };
enum : uint8_t {
    BIT_PROBE1 = 1u << 3,   // interior neighbour 1 of an equilibrium inlet: stores rho, ux
    BIT_PROBE2 = 1u << 4,   // interior neighbour 2: stores ux
    BIT_OUTUP = 1u << 5,    // upstream neighbour of an outlet: stores its incoming-direction f*
                            // (density-interpolated) or its moments (neighbour-equilibrium outlets)
    BIT_REFBULK = 1u << 6,  // reference flag == 1 (cells the error monitor sums over)
    BIT_SPONGE = 1u << 7,   // inside the outlet sponge: the relaxation rate is lowered
};
constexpr uint8_t CLS_MASK = 7;

// outlet kinds (the values of LBM_OUTLET_* in lbm.h)
constexpr int OUT_INTERPOLATED = 0, OUT_NEQ = 1, OUT_NEQ_OMEGA = 2, OUT_NEQ_OMEGA_RF = 3, OUT_DENSITY_EQ = 4;

// velocity set, lane types and collision math: lbm_math.cuh
// the 9 directions with c_x = -s (s = +1: outlet facing +x) as used by the outlet side table
LBM_HD constexpr int outlet_slot(int v) {  // k of direction v among the 9 with the same c_x
    constexpr int t[27] = {-1, 0, 0, -1, -1, -1, -1, 1, 1, 2, 2, 3, 3, -1, -1, 4, 4, -1, -1, 5, 5, 6, 6, 7, 7, 8, 8};
    return t[v];
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
    float tauf, cles18f, nuf, Ff[3];  // the same in FP32 (no FP64 instruction on the FP32 path)
    double omega0;           // 1/tau
    float omega0f;
    int has_force;
    float rho0, scale, inv_scale;  // FP16-deviation encoding
    int f16_sr;              // FP16 stores round stochastically (else to nearest)
    uint32_t sr_step_seed;   // step_seed(m)
    float raw_rho, raw_mdiag;  // sum_v w_v rho0 and sum_v w_v rho0 c_vx^2 of the FP16 codec's references
    uint32_t sr_mul, sr_add; // packed FP16 stores: seed = hash * sr_mul + sr_add (sr_seed_pair)
    uint32_t sr_off[27];     // packed FP16 stores: rounding bits of direction v = seed + sr_off[v]
                             // (v kSrWeyl when rounding stochastically, 0 when to nearest)
    float wr[27];            // w_v rho0            (decode f = h 2^-s + w_v rho0)
    float nwrs[27];          // -w_v rho0 2^s       (encode h = f 2^s - w_v rho0 2^s)
    float2 wr2[27], nwrs2[27];  // the same as (x, x) pairs for the packed two-cell path
    float2 scale2, inv_scale2;
    // byte addresses of the 27 slot arrays for bulk cells off the periodic seams:
    // element = base + idx
    unsigned long long rd_even[27];  // A[v]                  (even read of direction v)
    unsigned long long rd_odd[27];   // A[opp v] - off(c_v)   (odd read: cell x - c_v)
    unsigned long long wr_even[27];  // A[opp v]              (even write of f*_v)
    unsigned long long wr_odd[27];   // A[v] + off(c_v)       (odd write: cell x + c_v)
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
    int outlet_kind;         // LBM_OUTLET_*
    void* out_msave;         // [2][4][n_ms] of S::R : parity, {rho, ux, uy, uz}, cell (neighbour-equilibrium)
    const int32_t* out_nb;   // [9][n_out] : out_msave entry of the cell x + c_v, per entering direction
    int n_ms;
    int inlet_zouhe;         // flag -1 nodes follow InletVelocityZouHe (else the moving wall)
    // symmetry nodes (half-way specular reflection across a +-y plane)
    const int32_t* sym_dir;  // [n_sym] : +1 normal +y, -1 normal -y
    int n_sym;
    // outlet sponge: cells with BIT_SPONGE relax with omega - slope * (coordinate - begin)
    int sponge_axis, sponge_begin;
    double sponge_slope;
    float sponge_slopef;
    // learned closure (LBM_CLOSURE_MLP): fragment table [kMlpFragRows][32] and input normalisation
    const uint4* mlp_frag;
    MlpNorm mlp;
    __half* nut;             // per-cell nu_t of the last network evaluation (refresh interval > 1)
    int mlp_run;             // with nut: the network runs in this step
    int mlp_tc;              // the plain-row kernel evaluates the network with tcgen05.mma (TMEM)
    // per-step options
    double* acc;             // time-average accumulators [10][N] (nullptr: off)
    int* err;                // device error word (bounded waits that gave up)
};

// scalar parameters in the compute type
template <class R> LBM_D R p_tau(const Params& p) { if constexpr (std::is_same<R, float>::value) return p.tauf; else return p.tau; }
template <class R> LBM_D R p_cles18(const Params& p) { if constexpr (std::is_same<R, float>::value) return p.cles18f; else return p.cles18; }
template <class R> LBM_D R p_nu(const Params& p) { if constexpr (std::is_same<R, float>::value) return p.nuf; else return p.nu; }
template <class R> LBM_D R p_F(const Params& p, int a) { if constexpr (std::is_same<R, float>::value) return p.Ff[a]; else return p.F[a]; }

// ---- stochastic rounding of FP16 stores ---------------------------------------------------------------
// A value is rounded up or down to a neighbouring FP16 number with probability proportional to its
// distance to the other one, so increments far below one FP16 step (a body force of 1e-8 per step
// against a step of ~1e-5 in f) survive in expectation instead of being rounded away every time.
// Method: add 13 random bits below the FP16 mantissa of the FP32 bit pattern (23 - 10 = 13 bits are
// dropped) and truncate toward zero; unbiased for results in the FP16 normal range.  The random bits
// are a function of (element, step) only, so runs, resumes and kernel variants are reproducible.
// Hash: the "lowbias32" 32-bit integer finaliser (C. Wellons, hash-prospector).
LBM_HD uint32_t mix32(uint32_t h) {
    h ^= h >> 16; h *= 0x7FEB352Du;
    h ^= h >> 15; h *= 0x846CA68Bu;
    h ^= h >> 16;
    return h;
}
LBM_D uint32_t sr_seed(unsigned long long e, int m) {
    return mix32((uint32_t)e ^ mix32((uint32_t)m * 0x9E3779B9u + (uint32_t)(e >> 32)));
}
// the step's part of sr_seed for indices below 2^32 (the packed paths' pair indices), hashed once per
// launch on the host: sr_seed(e, m) == mix32(e ^ step_seed(m)) for such e
LBM_HD uint32_t step_seed(int m) { return mix32((uint32_t)m * 0x9E3779B9u); }
// The packed paths draw one 32-bit seed per pair (or per cell) from this hash and give direction v the
// bits seed + v K (K = kSrWeyl, a Weyl sequence: additions on the integer ALU pipe; an integer
// multiply per direction would compete with the collision's FP32 work for the FMA pipe, which bounds
// the FP16 step).  Every field of seed + v K is uniform when the seed is, so each rounding stays
// unbiased; the 27 directions of a pair get evenly spread dithers.  Round-to-nearest takes the same
// instructions: seed = hash * 0 + kHalfStep2x (Params::sr_mul, sr_add) and offsets sr_off[v] = 0.
constexpr uint32_t kSrWeyl = 0x9E3779B9u;
constexpr uint32_t kHalfStep2x = (0x1000u << 16) | 0x1000u;  // a half step in both cvt.rs fields
LBM_D uint32_t sr_seed_pair(uint32_t e, const Params& p) { return mix32(e ^ p.sr_step_seed) * p.sr_mul + p.sr_add; }
LBM_D __half half_sr(float v, uint32_t r13) { return __float2half_rz(__uint_as_float(__float_as_uint(v) + r13)); }
// the same dither with a fixed half step instead of random bits rounds to nearest (ties away from zero)
constexpr uint32_t kHalfStep13 = 0x1000u;  // for half_sr
// Packed stores: cvt.rs.f16x2.f32 (sm_100 family) rounds both values stochastically in one instruction,
// adding the 13-bit fields rbits[28:16] (upper half) and rbits[12:0] (lower half) below the FP16
// mantissa of the FP32 patterns and truncating: the method of half_sr (the field layout was measured
// on a GB300 against a software model, bit for bit on 65,536 inputs).
LBM_D __half2 half2_sr(float2 v, uint32_t r) {
    uint32_t h;
    asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(h) : "f"(v.y), "f"(v.x), "r"(r));  // upper v.y, lower v.x
    return *reinterpret_cast<__half2*>(&h);
}

// ---- population codecs ------------------------------------------------------------------------------
template <class S>
struct Codec;
template <>
struct Codec<StF64> {
    template <int V> LBM_D static double dec(const double* a, const Params&) { return *a; }
    template <int V> LBM_D static void enc(double* a, double v, const Params&) { *a = v; }
};
template <>
struct Codec<StF32> {
    template <int V> LBM_D static float dec(const float* a, const Params&) { return __ldg(a); }
    template <int V> LBM_D static void enc(float* a, float v, const Params&) { *a = v; }
};
template <>
struct Codec<StF16> {
    // f = w_v rho0 + h 2^-s, stored h = (f - w_v rho0) 2^s  (the FP16-deviation encoding)
    template <int V> LBM_D static float dec(const __half* a, const Params& p) {
        return fmaf(__half2float(__ldg(a)), p.inv_scale, p.wr[V]);
    }
    template <int V> LBM_D static void enc(__half* a, float v, const Params& p) {
        const float e = fmaf(v, p.scale, p.nwrs[V]);
        const uint32_t r = sr_seed((unsigned long long)(a - (const __half*)p.f), p.m) >> 19;
        *a = half_sr(e, p.f16_sr ? r : kHalfStep13);
    }
};

// ---- equilibrium (second-order polynomial of the reference, e.g. OmegaLES.h:47-66) ----------
template <int V, class R>
LBM_D R feq(R r, R ux, R uy, R uz, R u2) {
    const R cu = V == 0 ? (R)0 : cdotu<V>(ux, uy, uz);
    return (R)wgt(V) * r * ((R)1 + (R)3 * cu + (R)4.5 * cu * cu - (R)1.5 * u2);
}

// ---- cell geometry: wrapped neighbour coordinates (general path) ----------------------------------
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
// true when a neighbour index of (x,y,z) wraps across a periodic seam
LBM_D bool on_seam(const Params& p, int x, int y, int z) {
    return (p.wrap[0] && (x == 0 || x == p.nx - 1)) || (p.wrap[1] && (y == 0 || y == p.ny - 1)) ||
           (p.wrap[2] && (z == 0 || z == p.nz - 1));
}

// level of a 3-level side table for step index k (k may be -1 or -2)
LBM_D int lvl3(int k) { return ((k % 3) + 3) % 3; }

template <class S, int V>
LBM_D typename S::R load_at(const Params& p, long long e) {
    return Codec<S>::template dec<V>((const typename S::T*)p.f + e, p);
}
template <class S, int V>
LBM_D void store_at(const Params& p, long long e, typename S::R v) {
    Codec<S>::template enc<V>((typename S::T*)p.f + e, v, p);
}

// ---- fast path: bulk cells off the seams ----------------------------------------------------------
template <class S, bool ODD>
LBM_D void load_fast(const Params& p, unsigned idx, typename S::R (&f)[27]) {
    using T = typename S::T;
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        // ODD reads slot opp(V) of cell x - c_V; even reads slot V of the cell itself
        const T* a = (const T*)(ODD ? p.rd_odd[V] : p.rd_even[V]) + idx;
        f[V] = Codec<S>::template dec<ODD ? opp(V) : V>(a, p);
    });
}
template <class S, bool ODD>
LBM_D void store_fast(const Params& p, unsigned idx, const typename S::R (&f)[27]) {
    using T = typename S::T;
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        T* a = (T*)(ODD ? p.wr_odd[V] : p.wr_even[V]) + idx;
        Codec<S>::template enc<ODD ? V : opp(V)>(a, f[V], p);
    });
}

// ---- gather: the pre-collision populations df_m(x, .) of a non-solid, non-inlet cell ----------
// DRAG: accumulate the momentum-exchange force over solid links (read-only kernels only).
template <class S, bool ODD, bool DRAG>
LBM_D void gather(const Params& p, const Cell& c, int cl, typename S::R (&f)[27], typename S::R (&drag)[3]) {
    using R = typename S::R;
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
            if (ODD) f[V] = load_at<S, opp(V)>(p, opp(V) * N + nbr<-cx(V), -cy(V), -cz(V)>(c));
            else     f[V] = load_at<S, V>(p, V * N + c.idx);
        });
        return;
    }
    // EDGE, OUTLET or SYM, m >= 1: per-link rules
    const int osgn = (cl == CLS_OUTLET) ? p.out_dir[p.aux[c.idx]] : 0;
    const int ysgn = (cl == CLS_SYM) ? p.sym_dir[p.aux[c.idx]] : 0;
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        if (osgn != 0 && cx(V) == -osgn) { f[V] = (R)0; return; }  // outlet rule below
        if (nbr_oob<-cx(V), -cy(V), -cz(V)>(c)) {  // a link from outside the box (rejected at set-up)
            f[V] = (R)0;
            return;
        }
        const long long nb = nbr<-cx(V), -cy(V), -cz(V)>(c);
        const int ncl = p.cls[nb] & CLS_MASK;
        if (ncl == CLS_SOLID) {
            // half-way bounce-back: f_v(x) = f*_{opp v}(x) of the previous step
            R b = ODD ? load_at<S, V>(p, V * N + c.idx) : load_at<S, opp(V)>(p, opp(V) * N + nb);
            f[V] = b;
            // fluid momentum lost through the link: b*c_{opp v} - b*c_v = -2 b c_v (not on the links a
            // symmetry node takes from across its plane)
            if (DRAG && !(cy(V) != 0 && cy(V) == -ysgn)) {
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
            const R nu3 = p_nu<R>(p) / (R)3;
            R rb;
            if (p.in_dir[id] > 0) rb = r1 + nu3 * ((ux1 - ux2) - (ub0 - ux1));
            else                  rb = r1 + nu3 * ((ux1 - ub0) - (ux2 - ux1));
            f[V] = feq<V>(rb, ub0, ub1, ub2, ub0 * ub0 + ub1 * ub1 + ub2 * ub2);
        } else {
            if (ODD) f[V] = load_at<S, opp(V)>(p, opp(V) * N + nb);
            else     f[V] = load_at<S, V>(p, V * N + c.idx);
        }
    });
    if (ysgn != 0) {
        // BounceSymmetryHalf.h:84-131: a link entering across the plane (c_y = -sign of the normal; the
        // loop above bounced it back from the solid cell across) carries f*_{sym v} of the in-plane cell
        // s = x - (c_x, 0, c_z) from the previous step, sym mirroring c_y; a solid s keeps the bounce-back.
        // The value sits where s streamed it: after an even step in s's own slot opp(sym v), after an
        // odd one in slot sym v of the solid cell across the plane.
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            if constexpr (cy(V) != 0) {
                if (cy(V) == -ysgn) {
                    constexpr int SV = vid(cx(V), -cy(V), cz(V));
                    const long long sc = nbr<-cx(V), 0, -cz(V)>(c);
                    if ((p.cls[sc] & CLS_MASK) != CLS_SOLID)
                        f[V] = ODD ? load_at<S, opp(SV)>(p, opp(SV) * N + sc) : load_at<S, SV>(p, SV * N + nbr<0, -cy(V), 0>(c));
                }
            }
        });
    }
    if (osgn != 0 && p.outlet_kind != OUT_INTERPOLATED) {
        // values kept by the node in the previous step: g_v = f_eq_v(u, rho_b) (- f*_v for the
        // neighbour-equilibrium outlets, which then add f_eq_v of the cell x + c_v)
        const int id = p.aux[c.idx];
        const R* sv = (const R*)p.out_save + (long long)((p.m - 1) & 1) * 18 * p.n_out;
        const R* ms = (const R*)p.out_msave + (long long)((p.m - 1) & 1) * 4 * p.n_ms;
        const bool neq = p.outlet_kind != OUT_DENSITY_EQ;
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            if constexpr (cx(V) != 0) {
                if (cx(V) == -osgn) {
                    const int k = outlet_slot(V);
                    R g = sv[(9 + k) * p.n_out + id];
                    if (neq) {
                        const int e = p.out_nb[k * p.n_out + id];
                        const R r = ms[e], ux = ms[p.n_ms + e], uy = ms[2 * p.n_ms + e], uz = ms[3 * p.n_ms + e];
                        g += feq<V>(r, ux, uy, uz, ux * ux + uy * uy + uz * uz);
                    }
                    f[V] = g;
                }
            }
        });
    } else if (osgn != 0) {
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

// general scatter of the post-collision populations (EDGE/OUTLET cells, seams)
template <class S, bool ODD>
LBM_D void scatter(const Params& p, const Cell& c, const typename S::R (&f)[27]) {
    const long long N = p.N;
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        if (ODD) {
            if (!nbr_oob<cx(V), cy(V), cz(V)>(c)) store_at<S, V>(p, V * N + nbr<cx(V), cy(V), cz(V)>(c), f[V]);
        } else {
            store_at<S, opp(V)>(p, opp(V) * N + c.idx, f[V]);
        }
    });
}

// state df_m of an equilibrium-inlet node: f_eq(u_b, rho_b) with rho_b from the probe moments of
// step m-1 (InletVelocityEquilibrium.h:71-97 run at the end of step m-1)
template <class S>
LBM_D void inlet_state(const Params& p, const Cell& c, typename S::R (&f)[27]) {
    using R = typename S::R;
    const int id = p.aux[c.idx];
    const R* pr = (const R*)p.in_probe + (long long)lvl3(p.m - 1) * 3 * p.n_in;
    const R r1 = pr[id], ux1 = pr[p.n_in + id], ux2 = pr[2 * p.n_in + id];
    const R ub0 = p.in_u[id], ub1 = p.in_u[p.n_in + id], ub2 = p.in_u[2 * p.n_in + id];
    const R nu3 = p_nu<R>(p) / (R)3;
    R rb;
    if (p.in_dir[id] > 0) rb = r1 + nu3 * ((ux1 - ux2) - (ub0 - ux1));
    else                  rb = r1 + nu3 * ((ux1 - ub0) - (ux2 - ux1));
    const R u2 = ub0 * ub0 + ub1 * ub1 + ub2 * ub2;
    sfor<0, 27>([&](auto vc) { constexpr int V = decltype(vc)::value; f[V] = feq<V>(rb, ub0, ub1, ub2, u2); });
}

// ---- moments of a gathered cell for the read-only kernels ------------------------------------------
// rho and u as the reference's moment pass defines them (MomentDensityVelocityN27.h:65-81),
// with the half-force velocity shift
template <class R>
LBM_D void moments(const R (&f)[27], const Params& p, R& rho, R& jx, R& jy, R& jz, R& ux, R& uy, R& uz) {
    const Mom<R> m = raw_moments(f);
    rho = m.rho; jx = m.jx; jy = m.jy; jz = m.jz;
    const R ri = rcp(rho);
    ux = (jx + (R)0.5 * p_F<R>(p, 0)) * ri;
    uy = (jy + (R)0.5 * p_F<R>(p, 1)) * ri;
    uz = (jz + (R)0.5 * p_F<R>(p, 2)) * ri;
}

}  // namespace lbm
