// lbm_oracle.cpp - CPU ORACLE of the stloufra/LB D3Q27 solver step.  TEST INFRASTRUCTURE ONLY.
//
// This file restates, hook by hook and in the reference's own pass structure (separate
// omega, collision, A-B streaming, sparse-list boundary and moment passes), the algorithm of
// the reference solver so that the GPU kernels of this repository can be checked against it.
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the
// product library never does.  Citations are paths inside the reference project.
//
// Parity anchoring: the reference publishes no solver outputs (no tests, no committed fields),
// so the solver part of this oracle is "parity unpinned" by reference data; it is pinned only
// by reading the reference code and by known-answer properties (equilibrium is a fixed point,
// mass/momentum conservation, ghost-plane periodic == index wrap).  The voxelizer part
// (voxel_oracle.cpp) is pinned by the reference's committed golden mesh file.
//
// Reference defects reproduced only when ref_compat != 0:
//   * c_rev[20] = 21 instead of 19 (models/D3Q27/D3Q27.h:120-124);
//   * wall nodes need > 2 on the wall-pass count, i.e. >= 2 solid neighbours
//     (geometry/geometryMesherBoundary.h:459), so single-corner-contact cells are skipped;
//   * ErrorQuadratic's z term uses uStat.y - uErr.z (errorEvaluations/ErrorQuadratic.h:43-44);
//   * cumulant-2017: the third-order limiter arguments, the bulk reference and eq. 44's gradient
//     term (solvers/collisions/CollisionCumD3Q27Turbulent2017.h:256-266, :295, :351).
//
// Extensions with no reference counterpart (off unless requested): body force (Guo term for
// SRT, velocity shift for the cumulant, where G2015 eq. 85-87 carry it), native index-wrap
// periodicity (the reference uses ghost planes, Periodic.h; equivalence is tested), FP64
// time-average accumulators with <u_i u_j>.

#include "../include/lbm.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ---- D3Q27 tables: models/D3Q27/D3Q27.h:81-124 ------------------------------------------
static const int C[27][3] = {
    {0, 0, 0},
    {1, 0, 0},   {-1, 0, 0},  {0, 0, -1},  {0, 0, 1},   {0, -1, 0},  {0, 1, 0},
    {1, 0, -1},  {-1, 0, 1},  {1, 0, 1},   {-1, 0, -1}, {-1, -1, 0}, {1, 1, 0},
    {0, 1, -1},  {0, -1, 1},  {-1, 1, 0},  {1, -1, 0},  {0, 1, 1},   {0, -1, -1},
    {-1, 1, -1}, {1, -1, 1},  {-1, -1, 1}, {1, 1, -1},  {1, -1, -1}, {-1, 1, 1},
    {-1, -1, -1}, {1, 1, 1}};
// weights 8/27, 2/27, 1/54, 1/216 (D3Q27.h:113-118)
static double weight(int v) {
    int n = std::abs(C[v][0]) + std::abs(C[v][1]) + std::abs(C[v][2]);
    return n == 0 ? 8.0 / 27.0 : n == 1 ? 2.0 / 27.0 : n == 2 ? 1.0 / 54.0 : 1.0 / 216.0;
}
static const int CREV_OK[27] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14,
                                13, 16, 15, 18, 17, 20, 19, 22, 21, 24, 23, 26, 25};
static const int CREV_REF[27] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14,
                                 13, 16, 15, 18, 17, 20, 21, 22, 21, 24, 23, 26, 25};

// the y mirror of each direction: (c_x, -c_y, c_z).  The reference's c_sym_y (D3Q27.h:162-190) maps
// seven directions elsewhere; ref_compat uses its entries there.
static int sym_y_ok(int v) {
    for (int w = 0; w < 27; w++)
        if (C[w][0] == C[v][0] && C[w][1] == -C[v][1] && C[w][2] == C[v][2]) return w;
    return -1;
}
static int sym_y_ref(int v) {
    switch (v) {
        case 11: return 16; case 12: return 15; case 19: return 19; case 20: return 23;
        case 22: return 22; case 23: return 21; case 24: return 20;
        default: return sym_y_ok(v);
    }
}

template <class R>
struct Sim {
    int nx, ny, nz;
    size_t N;
    int wrap[3];
    int collision, closure, inlet_kind, outlet_kind, ref_compat;
    double dump_low, dump_high;
    R tau, nu, cles, F[3], cs;
    R w[27];
    const int* crev;

    std::vector<int32_t> mesh;
    std::vector<R> df, dfp, rho, u[3], omega, uerr[3];
    // a per-cell relaxation rate that replaces the closure pass of the next step (checking a closure
    // computed outside the oracle, e.g. the learned eddy viscosity, against the GPU step that fuses it)
    std::vector<R> omega_next;
    bool use_omega_next = false;
    std::vector<double> a_rho, a_u[3], a_uu[6];
    int64_t a_count = 0;
    bool a_on = false;
    double drag[3] = {0, 0, 0};
    int64_t step_count = 0;

    struct Wall { int x, y, z, regular; };
    struct Inlet { int x, y, z; R n[3], v[3]; int regular; };
    struct Outlet { int x, y, z; R n[3], density; int regular; };
    struct Per { int x, y, z; R n[3]; int idx, regular; };
    struct Sym { int x, y, z; R n[3]; int regular; };
    std::vector<Wall> walls;
    std::vector<Inlet> inlets;
    std::vector<Outlet> outlets;
    std::vector<Per> pers;
    std::vector<Sym> syms;

    Sim(const lbm_config& c, int refc) {
        nx = c.nx; ny = c.ny; nz = c.nz;
        N = (size_t)nx * ny * nz;
        for (int a = 0; a < 3; a++) wrap[a] = c.periodic[a];
        collision = c.collision; closure = c.closure; inlet_kind = c.inlet_kind; ref_compat = refc;
        outlet_kind = c.outlet_kind; dump_low = c.omega_dumping_low; dump_high = c.omega_dumping_high;
        nu = (R)c.nu;
        tau = c.tau > 0 ? (R)c.tau : (R)(3.0 * c.nu + 0.5);
        cles = (R)c.cles;
        for (int a = 0; a < 3; a++) F[a] = (R)c.force[a];
        cs = (R)1 / std::sqrt((R)3);                  // LBMConstants.h:103
        for (int v = 0; v < 27; v++) w[v] = (R)weight(v);
        crev = refc ? CREV_REF : CREV_OK;
        mesh.assign(N, 1);
        df.assign(27 * N, 0); dfp.assign(27 * N, 0);
        rho.assign(N, 0); omega.assign(N, 0);
        for (int a = 0; a < 3; a++) { u[a].assign(N, 0); uerr[a].assign(N, 0); }
    }

    inline size_t id(int i, int j, int k) const { return (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k); }
    // neighbour coordinate along one axis; wrap if periodic, else may leave the box
    inline int nb(int i, int d, int a) const {
        int n = a == 0 ? nx : a == 1 ? ny : nz;
        int r = i + d;
        if (wrap[a]) { if (r < 0) r += n; else if (r >= n) r -= n; }
        return r;
    }
    inline bool inside(int i, int j, int k) const {
        return i >= 0 && j >= 0 && k >= 0 && i < nx && j < ny && k < nz;
    }
    // flag lookup; cells outside a non-periodic box read as solid (the reference relies on a
    // solid outer layer there, "additional_factor ... at least 1", main.cu:90)
    inline int32_t mesh_at(int i, int j, int k) const { return inside(i, j, k) ? mesh[id(i, j, k)] : 0; }

    inline R feq(R ux, R uy, R uz, R r, int v) const {
        // f_equilibrium lambdas, e.g. OmegaLES.h:47-66
        R uc = (R)C[v][0] * ux + (R)C[v][1] * uy + (R)C[v][2] * uz;
        R u2 = ux * ux + uy * uy + uz * uz;
        return w[v] * r * ((R)1 + (R)3 * uc + (R)4.5 * uc * uc - (R)1.5 * u2);
    }

    // ---- wall list: geometryMesherBoundary.h:439-484 + compileBoundaryArrayWall :514-550
    // wall_mesh: the BounceBackWallHalfMesh policy, which bounces back on the cells of flag exactly 2
    // (BounceBackWallHalfMesh.h:38) instead of the list; corrected, both take every fluid cell with a
    // solid neighbour
    int wall_mesh = 0;
    void build_wall_list() {
        walls.clear();
        int thr = ref_compat ? 2 : 1;  // reference: > 2 (:459); corrected: any solid neighbour
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    int32_t m = mesh[id(i, j, k)];
                    bool on = (wall_mesh && ref_compat) ? m == 2 : m > thr;
                    if (on) walls.push_back({i, j, k, m > 10 ? 0 : 1});
                }
        // -2 nodes are not wall nodes in the reference (compileBoundaryArrayWall erases them,
        // geometryMesherBoundary.h:533-550), so their links from solid cells keep their old value;
        // corrected: symmetry nodes bounce back on those links
        if (!ref_compat)
            for (const Sym& sy : syms) walls.push_back({sy.x, sy.y, sy.z, 0});
    }

    // ---- InitializationEquilibriumConstVector.h:20-141 (lattice units) ------------------
    void init_equilibrium(R r0, const R u0[3]) {
        a_count = 0; a_on = false;
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < (long long)N; c++) {
            if (mesh[c] != 0) { rho[c] = r0; for (int a = 0; a < 3; a++) u[a][c] = u0[a]; }
            else { rho[c] = 0; for (int a = 0; a < 3; a++) u[a][c] = 0; }
        }
        for (auto& in : inlets) {  // inletVelocities :180-192
            size_t c = id(in.x, in.y, in.z);
            for (int a = 0; a < 3; a++) u[a][c] = in.v[a];
        }
        init_df_from_moments();
        step_count = 0;
    }
    // with a body force the velocity is defined as (j + F/2)/rho: refresh the moments of the initial
    // state so the first collision sees the same definition as every later one (force extension)
    void force_consistent_moments() {
        if (F[0] != 0 || F[1] != 0 || F[2] != 0) moment_update();
    }
    void init_df_from_moments() {  // init_df :194-209
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < (long long)N; c++) {
            for (int v = 0; v < 27; v++) {
                R f = mesh[c] != 0 ? feq(u[0][c], u[1][c], u[2][c], rho[c], v) : (R)0;
                df[v * N + c] = f; dfp[v * N + c] = f;
            }
        }
    }

    // ---- OmegaLES.h:69-131 ---------------------------------------------------------------
    void omega_les() {
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < (long long)N; c++) {
            if (mesh[c] == 0) continue;
            R ux = u[0][c], uy = u[1][c], uz = u[2][c], r = rho[c];
            R pi[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            for (int v = 0; v < 27; v++) {
                R fe = feq(ux, uy, uz, r, v);
                R d = df[v * N + c] - fe;
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) pi[a][b] += (R)(C[v][a] * C[v][b]) * d;
            }
            R PI = 0;
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) PI += pi[a][b] * pi[a][b];
            R rinv = (R)1 / r;
            R term = (R)18 * cles * rinv;
            PI = std::sqrt(PI);
            R tles = tau * (R)0.5 + (R)0.5 * std::sqrt(tau * tau + term * PI);
            omega[c] = (R)1 / tles;
        }
    }
    // ---- OmegaNo.h:34-42 ----------------------------------------------------------------
    void omega_no() {
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < (long long)N; c++)
            if (mesh[c] != 0) omega[c] = (R)1 / tau;
    }

    // ---- CollisionSRTTurbulent.h:56-75 (+ Guo forcing extension) -------------------------
    void collision_srt() {
        bool force = F[0] != 0 || F[1] != 0 || F[2] != 0;
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < (long long)N; c++) {
            if (mesh[c] == 0) continue;
            R ux = u[0][c], uy = u[1][c], uz = u[2][c], r = rho[c], om = omega[c];
            for (int v = 0; v < 27; v++) {
                R f = df[v * N + c];
                R out = f - (f - feq(ux, uy, uz, r, v)) * om;
                if (force) {
                    R cu = (R)C[v][0] * ux + (R)C[v][1] * uy + (R)C[v][2] * uz;
                    R s = 0;
                    for (int a = 0; a < 3; a++) {
                        R ua = a == 0 ? ux : a == 1 ? uy : uz;
                        s += ((R)3 * ((R)C[v][a] - ua) + (R)9 * cu * (R)C[v][a]) * F[a];
                    }
                    out += ((R)1 - (R)0.5 * om) * w[v] * s;
                }
                dfp[v * N + c] = out;
            }
        }
    }

    // ---- CollisionCumD3Q27Turbulent2015.h:32-518 -------------------------------------------
    // Chimera triplets: slot s in {0,1,2} holds the velocity component s-1.
    static inline void fwd3(R m, R z, R p, R uu, R& k0, R& k1, R& k2) {
        // G2015 eq. 43-45 (reference :86-178)
        k0 = (p + m) + z;
        k1 = (p - m) - uu * k0;
        k2 = (p + m) - (R)2 * uu * (p - m) + uu * uu * k0;
    }
    static inline void bwd3(R k0, R k1, R k2, R uu, R& m, R& z, R& p) {
        // G2015 eq. 88-96 (reference :389-485)
        z = k0 * ((R)1 - uu * uu) - (R)2 * uu * k1 - k2;
        m = (k0 * (uu * uu - uu) + k1 * ((R)2 * uu - (R)1) + k2) * (R)0.5;
        p = (k0 * (uu * uu + uu) + k1 * ((R)2 * uu + (R)1) + k2) * (R)0.5;
    }
    // G17 = false: CollisionCumD3Q27Turbulent2015 (all rates but omega_1 equal to 1);
    // G17 = true: CollisionCumD3Q27Turbulent2017.h:241-376 (limited third-order rates, fourth-order
    // cumulants driven by the velocity gradients).  With ref_compat the 2017 operator keeps two
    // reference defects: omega210p012 / omega210m012 are limited by C120 +- C102 instead of
    // C210 +- C012 (:256-266), the bulk part of Dxu subtracts (-1 + rho) instead of k000 (:295), and
    // eq. 44's gradient term is not the axis image of eq. 43's (:351).
    void cumulant_cell(size_t c, bool G17 = false, bool combined = false) {
        R f[3][3][3];
        for (int v = 0; v < 27; v++) f[C[v][0] + 1][C[v][1] + 1][C[v][2] + 1] = df[v * N + c];
        const R ux = u[0][c], uy = u[1][c], uz = u[2][c], r = rho[c], omg = omega[c];
        R a[3][3][3], b[3][3][3], k[3][3][3];
        for (int sx = 0; sx < 3; sx++)  // z pass
            for (int sy = 0; sy < 3; sy++)
                fwd3(f[sx][sy][0], f[sx][sy][1], f[sx][sy][2], uz, a[sx][sy][0], a[sx][sy][1], a[sx][sy][2]);
        for (int sx = 0; sx < 3; sx++)  // y pass
            for (int oz = 0; oz < 3; oz++)
                fwd3(a[sx][0][oz], a[sx][1][oz], a[sx][2][oz], uy, b[sx][0][oz], b[sx][1][oz], b[sx][2][oz]);
        for (int oy = 0; oy < 3; oy++)  // x pass
            for (int oz = 0; oz < 3; oz++)
                fwd3(b[0][oy][oz], b[1][oy][oz], b[2][oy][oz], ux, k[0][oy][oz], k[1][oy][oz], k[2][oy][oz]);
#define K(i, j, l) k[i][j][l]
        // central moments -> cumulants, G2015 eq. 47-54 (reference :188-232)
        const R C110 = K(1,1,0), C101 = K(1,0,1), C011 = K(0,1,1);
        const R C200 = K(2,0,0), C020 = K(0,2,0), C002 = K(0,0,2);
        const R C120 = K(1,2,0), C012 = K(0,1,2), C201 = K(2,0,1);
        const R C210 = K(2,1,0), C021 = K(0,2,1), C102 = K(1,0,2);
        const R C111 = K(1,1,1);
        const R C211 = K(2,1,1) - (K(2,0,0) * K(0,1,1) + (R)2 * K(1,0,1) * K(1,1,0)) / r;
        const R C121 = K(1,2,1) - (K(0,2,0) * K(1,0,1) + (R)2 * K(1,1,0) * K(0,1,1)) / r;
        const R C112 = K(1,1,2) - (K(0,0,2) * K(1,1,0) + (R)2 * K(0,1,1) * K(1,0,1)) / r;
        const R C220 = K(2,2,0) - (K(0,2,0) * K(2,0,0) + (R)2 * K(1,1,0) * K(1,1,0)) / r;
        const R C022 = K(0,2,2) - (K(0,0,2) * K(0,2,0) + (R)2 * K(0,1,1) * K(0,1,1)) / r;
        const R C202 = K(2,0,2) - (K(2,0,0) * K(0,0,2) + (R)2 * K(1,0,1) * K(1,0,1)) / r;
        const R C122 = K(1,2,2) - (K(0,2,0) * K(1,0,2) + K(0,0,2) * K(1,2,0) + (R)4 * K(0,1,1) * K(1,1,1) +
                                   (R)2 * (K(1,1,0) * K(0,1,2) + K(1,0,1) * K(0,2,1))) / r;
        const R C212 = K(2,1,2) - (K(0,0,2) * K(2,1,0) + K(2,0,0) * K(0,1,2) + (R)4 * K(1,0,1) * K(1,1,1) +
                                   (R)2 * (K(0,1,1) * K(2,0,1) + K(1,1,0) * K(1,0,2))) / r;
        const R C221 = K(2,2,1) - (K(2,0,0) * K(0,2,1) + K(0,2,0) * K(2,0,1) + (R)4 * K(1,1,0) * K(1,1,1) +
                                   (R)2 * (K(1,0,1) * K(1,2,0) + K(0,1,1) * K(2,1,0))) / r;
        const R C222 = K(2,2,2) - ((R)4 * K(1,1,1) * K(1,1,1) + K(2,0,0) * K(0,2,2) + K(0,2,0) * K(2,0,2) +
                                   K(0,0,2) * K(2,2,0) +
                                   (R)4 * (K(0,1,1) * K(2,1,1) + K(1,0,1) * K(1,2,1) + K(1,1,0) * K(1,1,2)) +
                                   (R)2 * (K(1,2,0) * K(1,0,2) + K(2,1,0) * K(0,1,2) + K(2,0,1) * K(0,2,1))) / r +
                  ((R)16 * K(1,1,0) * K(1,0,1) * K(0,1,1) +
                   (R)4 * (K(1,0,1) * K(1,0,1) * K(0,2,0) + K(0,1,1) * K(0,1,1) * K(2,0,0) +
                           K(1,1,0) * K(1,1,0) * K(0,0,2)) +
                   (R)2 * K(2,0,0) * K(0,2,0) * K(0,0,2)) / r / r;
        const R k000 = K(0,0,0), k100 = K(1,0,0), k010 = K(0,1,0), k001 = K(0,0,1);
#undef K
        // relaxation, G2015 eq. 55-73 (reference 2015 :240-316; 2017 :241-376)
        const R o1 = omg, o2 = 1, o6 = 1, o7 = 1, o8 = 1, o9 = 1, o10 = 1;
        R w120p102 = 1, w210p012 = 1, w201p021 = 1, w120m102 = 1, w210m012 = 1, w201m021 = 1, w111 = 1;
        R A4 = 0, B4 = 0;
        if (G17) {
            // G2017 eq. 14-16 and the limiter of its section 7 (lambda = 0.01)
            const R w3 = (R)8 * (o1 - (R)2) * (o2 * ((R)3 * o1 - (R)1) - (R)5 * o1) /
                         ((R)8 * ((R)5 - (R)2 * o1) * o1 + o2 * ((R)8 + o1 * ((R)9 * o1 - (R)26)));
            const R w4 = (R)8 * (o1 - (R)2) * (o1 + o2 * ((R)3 * o1 - (R)7)) /
                         (o2 * ((R)56 - (R)42 * o1 + (R)8 * o1 * o1) - (R)8 * o1);
            const R w5 = (R)24 * (o1 - (R)2) *
                         ((R)4 * o1 * o1 + o1 * o2 * ((R)18 - (R)13 * o1) + o2 * o2 * ((R)2 + o1 * ((R)6 * o1 - (R)11))) /
                         ((R)16 * o1 * o1 * (o1 - (R)6) - (R)2 * o1 * o2 * ((R)216 + (R)5 * o1 * ((R)9 * o1 - (R)46)) +
                          o2 * o2 * (o1 * ((R)3 * o1 - (R)10) * ((R)15 * o1 - (R)28) - (R)48));
            const R lam = (R)0.01;
            auto lim = [&](R w, R cc) { const R a = std::fabs(cc); return w + ((R)1 - w) * a / (r * lam + a); };
            w120p102 = lim(w3, C120 + C102);
            w210p012 = lim(w3, ref_compat ? C120 + C102 : C210 + C012);
            w201p021 = lim(w3, C201 + C021);
            w120m102 = lim(w4, C120 - C102);
            w210m012 = lim(w4, ref_compat ? C120 - C102 : C210 - C012);
            w201m021 = lim(w4, C201 - C021);
            w111 = lim(w5, C111);
            const R den = (o1 - o2) * (o2 * ((R)2 + (R)3 * o1) - (R)8 * o1);
            A4 = ((R)4 * o1 * o1 + (R)2 * o1 * o2 * (o1 - (R)6) + o2 * o2 * (o1 * ((R)10 - (R)3 * o1) - (R)4)) / den;
            B4 = ((R)4 * o1 * o2 * ((R)9 * o1 - (R)16) - (R)4 * o1 * o1 - (R)2 * o2 * o2 * ((R)2 + (R)9 * o1 * (o1 - (R)2))) /
                 ((R)3 * den);
        }
        // the 2017 header writes - (-1 + rho) (:295), the combined header's 2017 copy - -(-1 - rho)
        // (CollisionCumD3Q27TurbulentCombined.h:295)
        const R bulk0 = (G17 && ref_compat) ? (combined ? r + (R)1 : r - (R)1) : k000;
        const R Dxu = -o1 * (R)0.5 / r * ((R)2 * C200 - C020 - C002) - o2 * (R)0.5 / r * (C200 + C020 + C002 - bulk0);
        const R Dyv = Dxu + (R)3 * o1 * (R)0.5 / r * (C200 - C020);
        const R Dzw = Dxu + (R)3 * o1 * (R)0.5 / r * (C200 - C002);
        const R DxvDyu = -(R)3 * o1 / r * C110, DxwDzu = -(R)3 * o1 / r * C101, DywDzv = -(R)3 * o1 / r * C011;
        const R S110 = ((R)1 - o1) * C110, S101 = ((R)1 - o1) * C101, S011 = ((R)1 - o1) * C011;
        const R E61 = ((R)1 - o1) * (C200 - C020) - (R)3 * r * ((R)1 - o1 * (R)0.5) * (ux * ux * Dxu - uy * uy * Dyv);
        const R E64 = ((R)1 - o1) * (C200 - C002) - (R)3 * r * ((R)1 - o1 * (R)0.5) * (ux * ux * Dxu - uz * uz * Dzw);
        const R E65 = k000 * o2 + ((R)1 - o2) * (C200 + C020 + C002) -
                      (R)3 * r * ((R)1 - o2 / (R)2) * (ux * ux * Dxu + uy * uy * Dyv + uz * uz * Dzw);
        const R S200 = (R)1 / (R)3 * (E61 + E64 + E65);
        const R S020 = (R)1 / (R)3 * (E64 - (R)2 * E61 + E65);
        const R S002 = (R)1 / (R)3 * (E61 - (R)2 * E64 + E65);
        // third order: sums and differences relax with their own rates (G2015 eq. 61-66, G2017 eq. 37-42)
        const R P1 = ((R)1 - w120p102) * (C120 + C102), P2 = ((R)1 - w210p012) * (C210 + C012),
                P3 = ((R)1 - w201p021) * (C201 + C021);
        const R M1 = ((R)1 - w120m102) * (C120 - C102), M2 = ((R)1 - w210m012) * (C210 - C012),
                M3 = ((R)1 - w201m021) * (C201 - C021);
        const R S120 = (R)0.5 * (P1 + M1), S102 = (R)0.5 * (P1 - M1);
        const R S210 = (R)0.5 * (P2 + M2), S012 = (R)0.5 * (P2 - M2);
        const R S201 = (R)0.5 * (P3 + M3), S021 = (R)0.5 * (P3 - M3);
        const R S111 = ((R)1 - w111) * C111;
        // fourth order (G2017 eq. 43-48; A = B = 0 in the 2015 operator)
        const R vis = (R)1 / o1 - (R)0.5;
        const R E43 = (R)2 / (R)3 * vis * o6 * A4 * r * (Dxu - (R)2 * Dyv + Dzw) + ((R)1 - o6) * (C220 - (R)2 * C202 + C022);
        // C220 + C202 - 2 C022 follows 2 Dxu - Dyv - Dzw under an axis relabelling (each C_abc
        // with two 2-indices tracks the gradients of those two axes), so the isotropic driving
        // term is Dyv + Dzw - 2 Dxu; the reference writes Dxu + Dyv - 2 Dzw (:351).
        const R D44 = ref_compat ? Dxu + Dyv - (R)2 * Dzw : Dyv + Dzw - (R)2 * Dxu;
        const R E44 = (R)2 / (R)3 * vis * o6 * A4 * r * D44 + ((R)1 - o6) * (C220 + C202 - (R)2 * C022);
        const R E45 = -(R)4 / (R)3 * vis * o7 * A4 * r * (Dxu + Dyv + Dzw) + ((R)1 - o7) * (C220 + C202 + C022);
        const R S220 = (R)1 / (R)3 * (E43 + E44 + E45);
        const R S202 = (R)1 / (R)3 * (-E43 + E45);
        const R S022 = (R)1 / (R)3 * (-E44 + E45);
        const R S211 = -(R)1 / (R)3 * vis * o8 * B4 * r * DywDzv + ((R)1 - o8) * C211;
        const R S121 = -(R)1 / (R)3 * vis * o8 * B4 * r * DxwDzu + ((R)1 - o8) * C121;
        const R S112 = -(R)1 / (R)3 * vis * o8 * B4 * r * DxvDyu + ((R)1 - o8) * C112;
        const R S221 = ((R)1 - o9) * C221, S212 = ((R)1 - o9) * C212, S122 = ((R)1 - o9) * C122;
        const R S222 = ((R)1 - o10) * C222;
        // cumulants -> central moments, G2015 eq. 81-87 (reference :322-380)
        R q[3][3][3];
#define Q(i, j, l) q[i][j][l]
        Q(0,0,0) = k000;
        Q(1,1,0) = S110; Q(1,0,1) = S101; Q(0,1,1) = S011;
        Q(2,0,0) = S200; Q(0,2,0) = S020; Q(0,0,2) = S002;
        Q(1,2,0) = S120; Q(0,1,2) = S012; Q(2,0,1) = S201;
        Q(2,1,0) = S210; Q(0,2,1) = S021; Q(1,0,2) = S102;
        Q(1,1,1) = S111;
        Q(1,0,0) = -k100; Q(0,1,0) = -k010; Q(0,0,1) = -k001;
        Q(2,1,1) = S211 + (Q(2,0,0) * Q(0,1,1) + (R)2 * Q(1,0,1) * Q(1,1,0)) / r;
        Q(1,2,1) = S121 + (Q(0,2,0) * Q(1,0,1) + (R)2 * Q(1,1,0) * Q(0,1,1)) / r;
        Q(1,1,2) = S112 + (Q(0,0,2) * Q(1,1,0) + (R)2 * Q(0,1,1) * Q(1,0,1)) / r;
        Q(2,2,0) = S220 + (Q(0,2,0) * Q(2,0,0) + (R)2 * Q(1,1,0) * Q(1,1,0)) / r;
        Q(0,2,2) = S022 + (Q(0,0,2) * Q(0,2,0) + (R)2 * Q(0,1,1) * Q(0,1,1)) / r;
        Q(2,0,2) = S202 + (Q(2,0,0) * Q(0,0,2) + (R)2 * Q(1,0,1) * Q(1,0,1)) / r;
        Q(1,2,2) = S122 + (Q(0,2,0) * Q(1,0,2) + Q(0,0,2) * Q(1,2,0) + (R)4 * Q(0,1,1) * Q(1,1,1) +
                           (R)2 * (Q(1,1,0) * Q(0,1,2) + Q(1,0,1) * Q(0,2,1))) / r;
        Q(2,1,2) = S212 + (Q(0,0,2) * Q(2,1,0) + Q(2,0,0) * Q(0,1,2) + (R)4 * Q(1,0,1) * Q(1,1,1) +
                           (R)2 * (Q(0,1,1) * Q(2,0,1) + Q(1,1,0) * Q(1,0,2))) / r;
        Q(2,2,1) = S221 + (Q(2,0,0) * Q(0,2,1) + Q(0,2,0) * Q(2,0,1) + (R)4 * Q(1,1,0) * Q(1,1,1) +
                           (R)2 * (Q(1,0,1) * Q(1,2,0) + Q(0,1,1) * Q(2,1,0))) / r;
        Q(2,2,2) = S222 + ((R)4 * Q(1,1,1) * Q(1,1,1) + Q(2,0,0) * Q(0,2,2) + Q(0,2,0) * Q(2,0,2) +
                           Q(0,0,2) * Q(2,2,0) +
                           (R)4 * (Q(0,1,1) * Q(2,1,1) + Q(1,0,1) * Q(1,2,1) + Q(1,1,0) * Q(1,1,2)) +
                           (R)2 * (Q(1,2,0) * Q(1,0,2) + Q(2,1,0) * Q(0,1,2) + Q(2,0,1) * Q(0,2,1))) / r -
                   ((R)16 * Q(1,1,0) * Q(1,0,1) * Q(0,1,1) +
                    (R)4 * (Q(1,0,1) * Q(1,0,1) * Q(0,2,0) + Q(0,1,1) * Q(0,1,1) * Q(2,0,0) +
                            Q(1,1,0) * Q(1,1,0) * Q(0,0,2)) +
                    (R)2 * Q(2,0,0) * Q(0,2,0) * Q(0,0,2)) / r / r;
#undef Q
        // back to populations: x pass, y pass, z pass (G2015 eq. 88-96)
        R g[3][3][3], h[3][3][3], o[3][3][3];
        for (int oy = 0; oy < 3; oy++)
            for (int oz = 0; oz < 3; oz++)
                bwd3(q[0][oy][oz], q[1][oy][oz], q[2][oy][oz], ux, g[0][oy][oz], g[1][oy][oz], g[2][oy][oz]);
        for (int sx = 0; sx < 3; sx++)
            for (int oz = 0; oz < 3; oz++)
                bwd3(g[sx][0][oz], g[sx][1][oz], g[sx][2][oz], uy, h[sx][0][oz], h[sx][1][oz], h[sx][2][oz]);
        for (int sx = 0; sx < 3; sx++)
            for (int sy = 0; sy < 3; sy++)
                bwd3(h[sx][sy][0], h[sx][sy][1], h[sx][sy][2], uz, o[sx][sy][0], o[sx][sy][1], o[sx][sy][2]);
        for (int v = 0; v < 27; v++) dfp[v * N + c] = o[C[v][0] + 1][C[v][1] + 1][C[v][2] + 1];
    }
    void collision_cum2015() {
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < (long long)N; c++)
            if (mesh[c] != 0) cumulant_cell((size_t)c);
    }
    void collision_cum2017() {
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < (long long)N; c++)
            if (mesh[c] != 0) cumulant_cell((size_t)c, true);
    }
    // CollisionCumD3Q27TurbulentCombined.h:1066-1084: flag 1 -> the 2015 operator, other flags -> 2017
    void collision_combined() {
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < (long long)N; c++)
            if (mesh[c] != 0) cumulant_cell((size_t)c, mesh[c] != 1, true);
    }
    void collide_all() {
        if (collision == LBM_COLLISION_SRT) collision_srt();
        else if (collision == LBM_COLLISION_CUMULANT2017) collision_cum2017();
        else if (collision == LBM_COLLISION_CUMULANT_COMBINED) collision_combined();
        else collision_cum2015();
    }

    // ---- StreamingAB.h:38-68 (+ index wrap) ------------------------------------------------
    void streaming_ab() {
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    size_t c = id(i, j, k);
                    int32_t m = mesh[c];
                    if (!(m > 0 || m == -2 || m == -3)) continue;
                    for (int v = 0; v < 27; v++) {
                        int a = nb(i, -C[v][0], 0), b = nb(j, -C[v][1], 1), e = nb(k, -C[v][2], 2);
                        int32_t mn = mesh_at(a, b, e);
                        if (mn > 0 || mn == -2 || mn == -3) df[v * N + c] = dfp[v * N + id(a, b, e)];
                        else if (mn == -1) df[v * N + c] = df[v * N + id(a, b, e)];
                    }
                }
    }

    // ---- BounceBackWallHalf.h:29-52 (+ momentum-exchange drag) ---------------------------
    void bounce_back_wall() {
        double d0 = 0, d1 = 0, d2 = 0;
#pragma omp parallel for reduction(+ : d0, d1, d2) schedule(static)
        for (long long e = 0; e < (long long)walls.size(); e++) {
            const Wall& wl = walls[e];
            size_t c = id(wl.x, wl.y, wl.z);
            for (int v = 0; v < 27; v++) {
                int a = nb(wl.x, -C[v][0], 0), b = nb(wl.y, -C[v][1], 1), g = nb(wl.z, -C[v][2], 2);
                if (mesh_at(a, b, g) == 0) {
                    R in = dfp[crev[v] * N + c];
                    df[v * N + c] = in;
                    // momentum the fluid loses through this link: in*c_crev - in*c_v
                    d0 += (double)in * (C[crev[v]][0] - C[v][0]);
                    d1 += (double)in * (C[crev[v]][1] - C[v][1]);
                    d2 += (double)in * (C[crev[v]][2] - C[v][2]);
                }
            }
        }
        drag[0] = d0; drag[1] = d1; drag[2] = d2;
    }

    // ---- InletVelocityMovingWall.h:31-55 ---------------------------------------------------
    void inlet_moving_wall() {
#pragma omp parallel for schedule(static)
        for (long long e = 0; e < (long long)inlets.size(); e++) {
            const Inlet& in = inlets[e];
            size_t c = id(in.x, in.y, in.z);
            for (int v = 0; v < 27; v++) {
                if (in.n[0] * C[v][0] + in.n[1] * C[v][1] + in.n[2] * C[v][2] > 0) {
                    df[crev[v] * N + c] = dfp[v * N + c] - (R)6 * w[v] * rho[c] *
                                          ((R)C[v][0] * in.v[0] + (R)C[v][1] * in.v[1] + (R)C[v][2] * in.v[2]);
                }
            }
        }
    }

    // ---- InletVelocityEquilibrium.h:51-103 (x normals only, as the reference) ----------
    void inlet_equilibrium() {
#pragma omp parallel for schedule(static)
        for (long long e = 0; e < (long long)inlets.size(); e++) {
            const Inlet& in = inlets[e];
            int i = in.x, j = in.y, k = in.z;
            size_t c = id(i, j, k);
            bool xp = in.n[0] == 1 && in.n[1] == 0 && in.n[2] == 0;
            bool xm = in.n[0] == -1 && in.n[1] == 0 && in.n[2] == 0;
            if (!xp && !xm) continue;  // "Not yet supported inlet." (:162-164)
            R rhob;
            if (xp) {
                R ux1 = u[0][id(i - 1, j, k)], ux2 = u[0][id(i - 2, j, k)];
                R duxb = in.v[0] - ux1, dux1 = ux1 - ux2;
                rhob = rho[id(i - 1, j, k)] + nu / (R)3 * (dux1 - duxb);
            } else {
                R ux1 = u[0][id(i + 1, j, k)], ux2 = u[0][id(i + 2, j, k)];
                R duxb = ux1 - in.v[0], dux1 = ux2 - ux1;
                rhob = rho[id(i + 1, j, k)] + nu / (R)3 * (duxb - dux1);
            }
            for (int v = 0; v < 27; v++) df[v * N + c] = feq(in.v[0], in.v[1], in.v[2], rhob, v);
        }
    }

    // ---- OutletDensityInterpolated.h:170-252 -----------------------------------------------
    void outlet_density_interpolated() {
#pragma omp parallel for schedule(static)
        for (long long e = 0; e < (long long)outlets.size(); e++) {
            const Outlet& ot = outlets[e];
            int i = ot.x, j = ot.y, k = ot.z;
            size_t c = id(i, j, k);
            bool xp = ot.n[0] == 1 && ot.n[1] == 0 && ot.n[2] == 0;
            bool xm = ot.n[0] == -1 && ot.n[1] == 0 && ot.n[2] == 0;
            if (!xp && !xm) continue;  // "Not yet supported outlet." (:248-250)
            if (xp && !ot.regular) {  // irregular nodes (:186-198), only on the +x branch
                for (int v = 0; v < 27; v++) {
                    int dy = nb(j, -C[v][1], 1), dz = nb(k, -C[v][2], 2);
                    if (mesh_at(i, dy, dz) == 0) df[v * N + c] = df[crev[v] * N + c];
                }
            }
            int iu = xp ? i - 1 : i + 1;
            for (int v = 0; v < 27; v++) {
                if (ot.n[0] * C[v][0] + ot.n[1] * C[v][1] + ot.n[2] * C[v][2] < 0)
                    df[v * N + c] = cs * dfp[v * N + id(iu, j, k)] + ((R)1 - cs) * dfp[v * N + c];
            }
            R r = 0, jx = 0, jy = 0, jz = 0;
            for (int v = 0; v < 27; v++) r += df[v * N + c];
            for (int v = 0; v < 27; v++) {
                R f = df[v * N + c];
                if (C[v][0]) jx += (R)C[v][0] * f;
                if (C[v][1]) jy += (R)C[v][1] * f;
                if (C[v][2]) jz += (R)C[v][2] * f;
            }
            R ux = jx / ot.density, uy = jy / ot.density, uz = jz / ot.density;
            for (int v = 0; v < 27; v++)
                df[v * N + c] = df[v * N + c] - feq(ux, uy, uz, r, v) + feq(ux, uy, uz, (R)1, v);
        }
    }

    // ---- OutletNeighbourEquilibriumOmega(RF)::outletOmega, :18-79 ----------------------------
    // omega -= (high - low) / width * (distance from the sponge's first plane) over the last
    // ceil(10 %) of the lattice along the first outlet's normal axis (always at the high end)
    void outlet_omega() {
        const Outlet& o0 = outlets[0];
        float n[3], pl[3];
        for (int a = 0; a < 3; a++) { n[a] = (float)o0.n[a]; pl[a] = std::fabs(std::fabs(n[a]) - 1.f); }
        const int dims[3] = {nx, ny, nz};
        int d01[3], dimA[3], beg[3];
        for (int a = 0; a < 3; a++) {
            d01[a] = (int)std::ceil((float)dims[a] * 0.1f);
            dimA[a] = (int)((float)d01[a] * std::fabs(n[a]) + (float)dims[a] * std::fabs(pl[a]));
            beg[a] = dims[a] - dimA[a];
        }
        const int interval = (int)std::fabs((float)d01[0] * n[0] + (float)d01[1] * n[1] + (float)d01[2] * n[2]);
        const R der = ((R)dump_high - (R)dump_low) / (R)interval;
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = beg[2]; k < nz; k++)
            for (int j = beg[1]; j < ny; j++)
                for (int i = beg[0]; i < nx; i++) {
                    const int pos = (int)((float)(i - beg[0]) * n[0] * n[0] + (float)(j - beg[1]) * n[1] * n[1] +
                                          (float)(k - beg[2]) * n[2] * n[2]);
                    omega[id(i, j, k)] = omega[id(i, j, k)] - der * (R)pos;
                }
    }

    // ---- InletVelocityZouHe.h:85-97 -------------------------------------------------------
    void inlet_zou_he() {
#pragma omp parallel for schedule(static)
        for (long long e = 0; e < (long long)inlets.size(); e++) {
            const Inlet& in = inlets[e];
            size_t c = id(in.x, in.y, in.z);
            for (int v = 0; v < 27; v++)
                if (in.n[0] * C[v][0] + in.n[1] * C[v][1] + in.n[2] * C[v][2] > 0) {
                    R fneq = dfp[v * N + c] - feq(u[0][c], u[1][c], u[2][c], rho[c], v);
                    df[crev[v] * N + c] = fneq + feq(in.v[0], in.v[1], in.v[2], rho[c], crev[v]);
                }
        }
    }

    // ---- OutletNeighbourEquilibrium.h:93-125 (RF: OutletNeighbourEquilibriumOmegaRF.h:151-155) ----
    // entering links f_v = f_eq_v(u, rho_b) + (f_eq_v - f_v)(x + c_v), f_v(x + c_v) being the
    // population that x itself streamed there: its non-equilibrium part enters with the opposite sign,
    // which damps it (with the same sign the outlet feeds each link its own last value, and a perturbed
    // duct diverges within 50 steps)
    void outlet_neighbour_equilibrium(bool rf) {
#pragma omp parallel for schedule(static)
        for (long long e = 0; e < (long long)outlets.size(); e++) {
            const Outlet& ot = outlets[e];
            size_t c = id(ot.x, ot.y, ot.z);
            R dens = ot.density;
            if (rf && u[0][c] < 0) dens = (R)((double)dens - 0.5 * (double)u[0][c] * (double)u[0][c] * (double)dens);
            for (int v = 0; v < 27; v++) {
                if (!(ot.n[0] * C[v][0] + ot.n[1] * C[v][1] + ot.n[2] * C[v][2] < 0)) continue;
                int a = nb(ot.x, C[v][0], 0), b = nb(ot.y, C[v][1], 1), g = nb(ot.z, C[v][2], 2);
                if (!ot.regular && !(mesh_at(a, b, g) > 0)) continue;
                size_t q = id(a, b, g);
                R fen = feq(u[0][q], u[1][q], u[2][q], rho[q], v);
                R fn = df[v * N + q];
                R fbc = feq(u[0][c], u[1][c], u[2][c], dens, v);
                df[v * N + c] = fbc + (fen - fn);
            }
        }
    }

    // ---- OutletDensityEquilibrium.h:57-70: entering links at f_eq(u, rho_b); the reference takes the
    // equilibrium of the outgoing direction v for slot c_rev[v] (:66), reproduced with ref_compat
    void outlet_density_equilibrium() {
#pragma omp parallel for schedule(static)
        for (long long e = 0; e < (long long)outlets.size(); e++) {
            const Outlet& ot = outlets[e];
            size_t c = id(ot.x, ot.y, ot.z);
            for (int v = 0; v < 27; v++)
                if (ot.n[0] * C[v][0] + ot.n[1] * C[v][1] + ot.n[2] * C[v][2] > 0)
                    df[crev[v] * N + c] = feq(u[0][c], u[1][c], u[2][c], ot.density, ref_compat ? v : crev[v]);
        }
    }

    // ---- BounceSymmetryHalf.h:84-131 (y normals; the x and z branches are commented out) ---------
    // links entering across the plane take f*_{sym v} of the in-plane cell s = x - (c_x, 0, c_z).
    // Irregular nodes: a solid s bounces back; with ref_compat also on every link whose in-plane
    // projection is solid (:127-130), and a -2 s gets the extra write df(s, sym(c_rev v)) = f*(s, c_rev v)
    // (:117-121), which races with s's own rule in the reference; here it runs after all rules.
    void symmetry_half() {
        std::vector<char> done(syms.size(), 0);
#pragma omp parallel for schedule(static)
        for (long long e = 0; e < (long long)syms.size(); e++) {
            const Sym& sy = syms[e];
            if (!(sy.n[0] == 0 && std::fabs((double)sy.n[1]) == 1 && sy.n[2] == 0)) continue;  // "Fail." (:158-161)
            done[e] = 1;
            size_t c = id(sy.x, sy.y, sy.z);
            for (int v = 0; v < 27; v++) {
                int a = nb(sy.x, -C[v][0], 0), g = nb(sy.z, -C[v][2], 2);
                int sv = ref_compat ? sym_y_ref(v) : sym_y_ok(v);
                bool across = sy.n[1] * C[v][1] < 0;
                if (sy.regular) {
                    if (across) df[v * N + c] = dfp[sv * N + id(a, sy.y, g)];
                    continue;
                }
                int32_t m = mesh_at(a, sy.y, g);
                if (m != 0) {
                    if (across) df[v * N + c] = dfp[sv * N + id(a, sy.y, g)];
                } else if (across || ref_compat) {
                    df[v * N + c] = dfp[crev[v] * N + c];
                }
            }
        }
        if (!ref_compat) return;
        for (size_t e = 0; e < syms.size(); e++) {
            const Sym& sy = syms[e];
            if (!done[e] || sy.regular) continue;
            for (int v = 0; v < 27; v++) {
                int a = nb(sy.x, -C[v][0], 0), g = nb(sy.z, -C[v][2], 2);
                if (sy.n[1] * C[v][1] < 0 && mesh_at(a, sy.y, g) == -2) {
                    size_t sc = id(a, sy.y, g);
                    df[sym_y_ref(crev[v]) * N + sc] = dfp[crev[v] * N + sc];
                }
            }
        }
    }

    // ---- Periodic.h:43-138 (ghost-plane form) ----------------------------------------------
    void periodic_ghost() {
#pragma omp parallel for schedule(static)
        for (long long e = 0; e < (long long)pers.size(); e++) {
            const Per& p = pers[e];
            int i = p.x, j = p.y, k = p.z;
            size_t c = id(i, j, k);
            int ax = (std::fabs((double)p.n[0]) == 1 && p.n[1] == 0 && p.n[2] == 0) ? 0
                   : (p.n[0] == 0 && std::fabs((double)p.n[1]) == 1 && p.n[2] == 0) ? 1
                   : (p.n[0] == 0 && p.n[1] == 0 && std::fabs((double)p.n[2]) == 1) ? 2 : -1;
            if (ax < 0) continue;  // "Fail." (:135-137)
            size_t src = ax == 0 ? id(p.idx, j, k) : ax == 1 ? id(i, p.idx, k) : id(i, j, p.idx);
            for (int v = 0; v < 27; v++) {
                R nc = p.n[0] * C[v][0] + p.n[1] * C[v][1] + p.n[2] * C[v][2];
                if (nc < 0) df[v * N + c] = df[v * N + src];
                if (!p.regular && nc <= 0) {
                    int a = nb(i, C[v][0], 0), b = nb(j, C[v][1], 1), g = nb(k, C[v][2], 2);
                    if (mesh_at(a, b, g) == 0) df[crev[v] * N + c] = dfp[v * N + c];
                }
            }
        }
    }

    // ---- MomentDensityVelocityN27.h:27-83 (+ half-force velocity shift) ------------------
    void moment_update() {
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < (long long)N; c++) {
            if (mesh[c] == 0) continue;
            R r = 0, jx = 0, jy = 0, jz = 0;
            for (int v = 0; v < 27; v++) r += df[v * N + c];
            for (int v = 0; v < 27; v++) {
                R f = df[v * N + c];
                if (C[v][0]) jx += (R)C[v][0] * f;
                if (C[v][1]) jy += (R)C[v][1] * f;
                if (C[v][2]) jz += (R)C[v][2] * f;
            }
            rho[c] = r;
            u[0][c] = (jx + (R)0.5 * F[0]) / r;
            u[1][c] = (jy + (R)0.5 * F[1]) / r;
            u[2][c] = (jz + (R)0.5 * F[2]) / r;
        }
    }

    // ---- MomentTimeAvg.h:27-47 (FP64 accumulators, + <u_i u_j>) ------------------------------
    void timeavg_add() {
#pragma omp parallel for schedule(static)
        for (long long c = 0; c < (long long)N; c++) {
            double x = u[0][c], y = u[1][c], z = u[2][c];
            a_rho[c] += rho[c];
            a_u[0][c] += x; a_u[1][c] += y; a_u[2][c] += z;
            a_uu[0][c] += x * x; a_uu[1][c] += y * y; a_uu[2][c] += z * z;
            a_uu[3][c] += x * y; a_uu[4][c] += x * z; a_uu[5][c] += y * z;
        }
        a_count++;
    }

    // ---- SolverTurbulentLES::runSimulation loop body, SolverTurbulentLES.h:186-226 --------
    void step() {
        if (use_omega_next) {
            for (size_t c = 0; c < N; c++) if (mesh[c] != 0) omega[c] = omega_next[c];
            use_omega_next = false;
        } else if (closure == LBM_CLOSURE_SMAGORINSKY) omega_les(); else omega_no();
        if (!outlets.empty() && (outlet_kind == LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA ||
                                 outlet_kind == LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA_RF))
            outlet_omega();
        collide_all();
        streaming_ab();
        bounce_back_wall();
        if (!inlets.empty()) {
            if (inlet_kind == LBM_INLET_MOVING_WALL) inlet_moving_wall();
            else if (inlet_kind == LBM_INLET_ZOU_HE) inlet_zou_he();
            else inlet_equilibrium();
        }
        if (!outlets.empty()) {
            if (outlet_kind == LBM_OUTLET_DENSITY_INTERPOLATED) outlet_density_interpolated();
            else if (outlet_kind == LBM_OUTLET_DENSITY_EQUILIBRIUM) outlet_density_equilibrium();
            else outlet_neighbour_equilibrium(outlet_kind == LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA_RF);
        }
        if (!syms.empty()) symmetry_half();
        if (!pers.empty()) periodic_ghost();
        moment_update();
        if (a_on) timeavg_add();
        step_count++;
    }

    // ---- ErrorQuadratic.h:33-91 -------------------------------------------------------------
    double error_evaluation() {
        double s1 = 0, s2 = 0;
#pragma omp parallel for reduction(+ : s1, s2) schedule(static)
        for (long long c = 0; c < (long long)N; c++) {
            if (mesh[c] != 1) continue;
            R dx = u[0][c] - uerr[0][c], dy = u[1][c] - uerr[1][c];
            R dz = ref_compat ? u[1][c] - uerr[2][c] : u[2][c] - uerr[2][c];
            R a1 = dx * dx + dy * dy + dz * dz;
            R a2 = u[0][c] * u[0][c] + u[1][c] * u[1][c] + u[2][c] * u[2][c];
            s1 += (double)std::sqrt(a1);
            s2 += (double)std::sqrt(a2);
        }
        for (int a = 0; a < 3; a++) uerr[a] = u[a];
        return std::sqrt(s1) / std::sqrt(s2);
    }

    void diag(lbm_diag* d) {
        double m = 0, p0 = 0, p1 = 0, p2 = 0, vmax = 0;
        long long bad = 0, nf = 0;
#pragma omp parallel for reduction(+ : m, p0, p1, p2, bad, nf) reduction(max : vmax) schedule(static)
        for (long long c = 0; c < (long long)N; c++) {
            int32_t fl = mesh[c];
            if (!(fl > 0 || fl == -2 || fl == -3)) continue;
            nf++;
            bool ok = true;
            for (int v = 0; v < 27; v++) ok = ok && std::isfinite((double)df[v * N + c]);
            if (!ok) bad++;
            m += rho[c];
            p0 += (double)rho[c] * u[0][c]; p1 += (double)rho[c] * u[1][c]; p2 += (double)rho[c] * u[2][c];
            double s = std::sqrt((double)u[0][c] * u[0][c] + (double)u[1][c] * u[1][c] + (double)u[2][c] * u[2][c]);
            vmax = std::max(vmax, s);
        }
        d->mass = m; d->momentum[0] = p0; d->momentum[1] = p1; d->momentum[2] = p2;
        for (int a = 0; a < 3; a++) d->drag[a] = drag[a];
        d->max_speed = vmax; d->nonfinite = bad; d->fluid_cells = nf; d->step = step_count;
    }
};

// ---- geometryMesherBoundary::meshingBoundaryWall, geometryMesherBoundary.h:439-484 --------
static void wall_pass(int32_t* m, int nx, int ny, int nz) {
    auto at = [&](int i, int j, int k) -> int32_t& { return m[(size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k)]; };
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                if (at(i, j, k) <= 0) continue;
                for (int l = -1; l <= 1; l++)
                    for (int mm = -1; mm <= 1; mm++)
                        for (int n = -1; n <= 1; n++) {
                            int a = i + l, b = j + mm, c = k + n;
                            if (a >= 0 && b >= 0 && c >= 0 && a < nx && b < ny && c < nz && at(a, b, c) == 0)
                                at(i, j, k) += 1;
                        }
            }
}

struct Handle {
    int prec;
    Sim<float>* s32 = nullptr;
    Sim<double>* s64 = nullptr;
};

}  // namespace orc

using namespace orc;

#define DISPATCH(h, ...)                                       \
    do {                                                       \
        if ((h)->prec == 32) { auto* S = (h)->s32; __VA_ARGS__; } \
        else { auto* S = (h)->s64; __VA_ARGS__; }              \
    } while (0)

extern "C" {

void* orc_create(const lbm_config* cfg, int precision, int ref_compat) {
    if (!cfg || cfg->nx <= 0 || cfg->ny <= 0 || cfg->nz <= 0) return nullptr;
    Handle* h = new Handle;
    h->prec = precision == 32 ? 32 : 64;
    if (h->prec == 32) h->s32 = new Sim<float>(*cfg, ref_compat);
    else h->s64 = new Sim<double>(*cfg, ref_compat);
    return h;
}
void orc_destroy(void* p) {
    Handle* h = (Handle*)p;
    if (!h) return;
    delete h->s32; delete h->s64; delete h;
}
void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
// host memory bandwidth (STREAM triad a = b + s c over n doubles per array, arrays first touched by the
// threads that use them, best of `reps`), in GB/s counting 24 bytes per element; reported beside the
// timed CPU baseline so its GLUPS can be read against the host's own roofline
double orc_host_stream_gbs(long long n, int reps) {
    std::vector<double> a((size_t)n), b((size_t)n), c((size_t)n);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; i++) { a[i] = 0.0; b[i] = 1.0; c[i] = 2.0; }
    double best = 0.0;
    for (int r = 0; r < reps; r++) {
        const double t0 = omp_get_wtime();
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < n; i++) a[i] = b[i] + 3.0 * c[i];
        const double dt = omp_get_wtime() - t0;
        if (dt > 0) best = std::max(best, 24.0 * (double)n / dt / 1e9);
    }
    return best + 0.0 * a[(size_t)(n / 2)];
}
int orc_set_flags(void* p, const int32_t* flags) {
    Handle* h = (Handle*)p;
    DISPATCH(h, { std::memcpy(S->mesh.data(), flags, S->N * sizeof(int32_t)); S->build_wall_list(); });
    return 0;
}
int orc_set_bc(void* p, const lbm_bc_inlet* in, int nin, const lbm_bc_outlet* out, int nout) {
    Handle* h = (Handle*)p;
    DISPATCH(h, {
        using SR = std::remove_pointer_t<decltype(S)>;
        S->inlets.clear(); S->outlets.clear(); S->syms.clear();
        S->build_wall_list();
        for (int e = 0; e < nin; e++) {
            typename SR::Inlet r;
            r.x = in[e].vertex.x; r.y = in[e].vertex.y; r.z = in[e].vertex.z;
            for (int a = 0; a < 3; a++) { r.n[a] = in[e].normal[a]; r.v[a] = in[e].velocity[a]; }
            r.regular = in[e].regular;
            S->inlets.push_back(r);
        }
        for (int e = 0; e < nout; e++) {
            typename SR::Outlet r;
            r.x = out[e].vertex.x; r.y = out[e].vertex.y; r.z = out[e].vertex.z;
            for (int a = 0; a < 3; a++) r.n[a] = out[e].normal[a];
            r.density = out[e].density; r.regular = out[e].regular;
            S->outlets.push_back(r);
        }
    });
    return 0;
}
int orc_set_wall_policy(void* p, int mesh_variant) {
    Handle* h = (Handle*)p;
    DISPATCH(h, { S->wall_mesh = mesh_variant; S->build_wall_list(); });
    return 0;
}
int orc_set_symmetry(void* p, const lbm_bc_symmetry* rec, int n) {
    Handle* h = (Handle*)p;
    DISPATCH(h, {
        using SR = std::remove_pointer_t<decltype(S)>;
        S->syms.clear();
        for (int e = 0; e < n; e++) {
            typename SR::Sym r;
            r.x = rec[e].vertex.x; r.y = rec[e].vertex.y; r.z = rec[e].vertex.z;
            for (int a = 0; a < 3; a++) r.n[a] = rec[e].normal[a];
            r.regular = rec[e].regular;
            S->syms.push_back(r);
        }
        S->build_wall_list();
    });
    return 0;
}
// periodic ghost-plane records: 8 int32 each (x, y, z, nx, ny, nz, periodicIndex, regular)
int orc_set_periodic_list(void* p, const int32_t* rec, int n) {
    Handle* h = (Handle*)p;
    DISPATCH(h, {
        using SR = std::remove_pointer_t<decltype(S)>;
        S->pers.clear();
        for (int e = 0; e < n; e++) {
            const int32_t* q = rec + 8 * e;
            typename SR::Per r;
            r.x = q[0]; r.y = q[1]; r.z = q[2];
            r.n[0] = q[3]; r.n[1] = q[4]; r.n[2] = q[5];
            r.idx = q[6]; r.regular = q[7];
            S->pers.push_back(r);
        }
    });
    return 0;
}
int orc_init_equilibrium(void* p, double rho0, const double* u0) {
    Handle* h = (Handle*)p;
    DISPATCH(h, {
        using RR = std::remove_reference_t<decltype(S->rho[0])>;
        RR uu[3] = {(RR)u0[0], (RR)u0[1], (RR)u0[2]};
        S->init_equilibrium((RR)rho0, uu);
        S->force_consistent_moments();
    });
    return 0;
}
// rho: N, u: 3N component-major (inlet nodes take their record velocity); then df = df_post = feq (init_df)
int orc_init_fields(void* p, const double* rho, const double* u) {
    Handle* h = (Handle*)p;
    DISPATCH(h, {
        for (size_t c = 0; c < S->N; c++) {
            if (S->mesh[c] != 0) {
                S->rho[c] = rho[c];
                for (int a = 0; a < 3; a++) S->u[a][c] = u[a * S->N + c];
            } else { S->rho[c] = 0; for (int a = 0; a < 3; a++) S->u[a][c] = 0; }
        }
        for (auto& in : S->inlets) {  // inletVelocities, InitializationEquilibriumVariables.h:140-154
            size_t c = S->id(in.x, in.y, in.z);
            for (int a = 0; a < 3; a++) S->u[a][c] = in.v[a];
        }
        S->init_df_from_moments();
        S->force_consistent_moments();
        S->step_count = 0;
    });
    return 0;
}
int orc_step(void* p, int n) {
    Handle* h = (Handle*)p;
    DISPATCH(h, { for (int s = 0; s < n; s++) S->step(); });
    return 0;
}
int orc_get_moments(void* p, double* rho, double* u) {
    Handle* h = (Handle*)p;
    DISPATCH(h, {
        for (size_t c = 0; c < S->N; c++) {
            if (rho) rho[c] = S->rho[c];
            if (u) for (int a = 0; a < 3; a++) u[a * S->N + c] = S->u[a][c];
        }
    });
    return 0;
}
int orc_get_omega(void* p, double* om) {
    Handle* h = (Handle*)p;
    DISPATCH(h, { for (size_t c = 0; c < S->N; c++) om[c] = S->omega[c]; });
    return 0;
}
int orc_set_omega_next(void* p, const double* om) {
    Handle* h = (Handle*)p;
    DISPATCH(h, {
        S->omega_next.resize(S->N);
        for (size_t c = 0; c < S->N; c++) S->omega_next[c] = om[c];
        S->use_omega_next = true;
    });
    return 0;
}
int orc_get_df(void* p, double* f) {
    Handle* h = (Handle*)p;
    DISPATCH(h, { for (size_t e = 0; e < 27 * S->N; e++) f[e] = S->df[e]; });
    return 0;
}
int orc_set_df(void* p, const double* f) {
    // sets the pre-collision populations and refreshes rho/u with the moment pass
    Handle* h = (Handle*)p;
    DISPATCH(h, { for (size_t e = 0; e < 27 * S->N; e++) S->df[e] = f[e]; S->moment_update(); });
    return 0;
}
int orc_timeavg_begin(void* p) {
    Handle* h = (Handle*)p;
    DISPATCH(h, {
        S->a_rho.assign(S->N, 0);
        for (int a = 0; a < 3; a++) S->a_u[a].assign(S->N, 0);
        for (int a = 0; a < 6; a++) S->a_uu[a].assign(S->N, 0);
        S->a_count = 0; S->a_on = true;
    });
    return 0;
}
int orc_timeavg_end(void* p) {
    Handle* h = (Handle*)p;
    DISPATCH(h, { S->a_on = false; });
    return 0;
}
// MomentTimeAvg::momentAvg (:49-80): divide by the count
int orc_timeavg_get(void* p, double* rho, double* u, double* uu, int64_t* count) {
    Handle* h = (Handle*)p;
    DISPATCH(h, {
        double n = S->a_count > 0 ? (double)S->a_count : 1.0;
        for (size_t c = 0; c < S->N; c++) {
            if (rho) rho[c] = S->a_rho.empty() ? 0 : S->a_rho[c] / n;
            if (u) for (int a = 0; a < 3; a++) u[a * S->N + c] = S->a_u[a].empty() ? 0 : S->a_u[a][c] / n;
            if (uu) for (int a = 0; a < 6; a++) uu[a * S->N + c] = S->a_uu[a].empty() ? 0 : S->a_uu[a][c] / n;
        }
        if (count) *count = S->a_count;
    });
    return 0;
}
int orc_error(void* p, double* err) {
    Handle* h = (Handle*)p;
    DISPATCH(h, { *err = S->error_evaluation(); });
    return 0;
}
int orc_diag(void* p, lbm_diag* d) {
    Handle* h = (Handle*)p;
    DISPATCH(h, { S->diag(d); });
    return 0;
}
int orc_wall_list_size(void* p) {
    Handle* h = (Handle*)p;
    int n = 0;
    DISPATCH(h, { n = (int)S->walls.size(); });
    return n;
}
void orc_mesher_wall_pass(int32_t* flags, int nx, int ny, int nz) { wall_pass(flags, nx, ny, nz); }
// one cumulant collision of a single cell of the given reference flag, for known-answer tests:
// f_in/f_out 27 doubles
void orc_collide_cell(int precision, int collision, const double* f_in, double rho, const double* u,
                      double omega, const double* force, double* f_out, int ref_compat, int flag) {
    lbm_config cfg;
    std::memset(&cfg, 0, sizeof(cfg));
    cfg.nx = cfg.ny = cfg.nz = 1; cfg.nu = 1.0 / 6.0; cfg.collision = collision;
    for (int a = 0; a < 3; a++) cfg.force[a] = force ? force[a] : 0.0;
    auto run = [&](auto* S) {
        S->mesh[0] = flag;
        for (int v = 0; v < 27; v++) S->df[v] = f_in[v];
        S->rho[0] = rho; for (int a = 0; a < 3; a++) S->u[a][0] = u[a];
        S->omega[0] = omega;
        S->collide_all();
        for (int v = 0; v < 27; v++) f_out[v] = S->dfp[v];
    };
    if (precision == 32) { Sim<float> S(cfg, ref_compat); run(&S); }
    else { Sim<double> S(cfg, ref_compat); run(&S); }
}

}  // extern "C"
