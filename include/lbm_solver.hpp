// lbm_solver.hpp - C++ host side of the solver: the reference's compile-time policy interface over the
// C ABI of lbm.h (header-only, C++17).
//
// The reference composes its solver from policy types (3D/simulation/src/solvers/SolverTurbulentLES.h:67-82)
// and owns its state in LBMConstants / LBMData (3D/simulation/src/data/LBMConstants.h:4-113,
// LBMData.h:3-77).  This header keeps those names: the same fourteen template parameters, tag types named
// after the reference's policies, and SolverTurbulentLES with initializeSimulation / runSimulation /
// probeWrite / convertToLattice.  A policy is a tag here, not a kernel: the whole step (omega, collision,
// streaming, boundaries, moments) is one fused kernel behind lbm_step, and the tags only select what it does.
// Policies the fused kernel does not implement fail to compile (static_assert) instead of running
// something else.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "lbm.h"

namespace lbm_gb300 {

// ---- policy tags (reference file of each in the comment) ----------------------------------------------
struct D3Q27 { static constexpr int numberOfDiscreteVelocities = 27; };           // models/D3Q27/D3Q27.h
struct CollisionCumD3Q27Turbulent2015 { static constexpr int32_t code = LBM_COLLISION_CUMULANT2015; static constexpr bool laminar = false; };
struct CollisionCumD3Q27Turbulent2017 { static constexpr int32_t code = LBM_COLLISION_CUMULANT2017; static constexpr bool laminar = false; };
struct CollisionCumD3Q27TurbulentCombined { static constexpr int32_t code = LBM_COLLISION_CUMULANT_COMBINED; static constexpr bool laminar = false; };
struct CollisionSRTTurbulent { static constexpr int32_t code = LBM_COLLISION_SRT; static constexpr bool laminar = false; };  // collisions/CollisionSRTTurbulent.h
// the laminar collisions relax with the global omega = 1/tau (Constants->omega:
// CollisionCumD3Q27Laminar.h:27, CollisionSRTLaminar.h:28, CollisionSRTunroll.h:27) and ignore the per-cell
// field, so the solver runs them with no closure and no outlet sponge whatever the other tags say
struct CollisionCumD3Q27Laminar { static constexpr int32_t code = LBM_COLLISION_CUMULANT2015; static constexpr bool laminar = true; };
struct CollisionSRTLaminar { static constexpr int32_t code = LBM_COLLISION_SRT; static constexpr bool laminar = true; };
struct CollisionSRTunroll { static constexpr int32_t code = LBM_COLLISION_SRT; static constexpr bool laminar = true; };  // CollisionSRTLaminar unrolled
struct OmegaLES { static constexpr int32_t code = LBM_CLOSURE_SMAGORINSKY; };      // turbulence/OmegaLES.h
struct OmegaNo { static constexpr int32_t code = LBM_CLOSURE_NONE; };             // turbulence/OmegaNo.h
struct OmegaMLP { static constexpr int32_t code = LBM_CLOSURE_MLP; };             // learned closure (no reference policy)
struct StreamingAB {};                     // streamings/StreamingAB.h (AA pattern in place here)
struct BounceBackWallHalf {};              // boundaryConditions/Wall/BounceBackWallHalf.h
struct BounceBackWallHalfMesh {};          // .../Wall/BounceBackWallHalfMesh.h (the same rule on every fluid cell)
struct NoSymmetry { static constexpr bool on = false; };           // boundaryConditions/Symmetry/NoSymmetry.h
struct BounceSymmetryHalf { static constexpr bool on = true; };    // boundaryConditions/Symmetry/BounceSymmetryHalf.h
struct Periodic { static constexpr bool on = true; };    // boundaryConditions/Periodic/Periodic.h (index wrap)
struct NoPeriodic { static constexpr bool on = false; };
struct InletVelocityMovingWall { static constexpr int32_t code = LBM_INLET_MOVING_WALL; };
struct InletVelocityEquilibrium { static constexpr int32_t code = LBM_INLET_EQUILIBRIUM; };
struct InletVelocityZouHe { static constexpr int32_t code = LBM_INLET_ZOU_HE; };  // Inlet/InletVelocityZouHe.h
// boundaryConditions/Outlet/*.h
struct OutletDensityInterpolated { static constexpr int32_t code = LBM_OUTLET_DENSITY_INTERPOLATED; };
struct OutletNeighbourEquilibrium { static constexpr int32_t code = LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM; };
struct OutletNeighbourEquilibriumOmega { static constexpr int32_t code = LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA; };
struct OutletNeighbourEquilibriumOmegaRF { static constexpr int32_t code = LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA_RF; };
struct OutletDensityEquilibrium { static constexpr int32_t code = LBM_OUTLET_DENSITY_EQUILIBRIUM; };
struct MomentDensityVelocityN27 {};        // moments/MomentDensityVelocityN27.h
struct MomentTimeAvg {};                   // moments/MomentTimeAvg.h
struct ErrorQuadratic {};                  // errorEvaluations/ErrorQuadratic.h
struct InitializationEquilibriumConstVector {};  // initializations/InitializationEquilibriumConstVector.h
// initializations/InitializationEquilibriumVariables.h: restart from the lattice-unit VTK dump
// <results_dir or "results">/<InitFileName> (lbm_vtk_read_variables)
struct InitializationEquilibriumVariables {};

// ---- state carriers (the fields of LBMConstants / LBMData this path uses) ------------------------------
struct LBMConstants {
    int dimX_int = 0, dimY_int = 0, dimZ_int = 0;
    double ny = 1.0 / 6.0;            // lattice kinematic viscosity
    double tau = 0.0;                 // > 0 overrides 3 ny + 1/2
    double CLES = 0.173;              // LBMConstants.h:70
    double Fx = 0.0, Fy = 0.0, Fz = 0.0;
    double rho0 = 1.0;
    double VelocityInit[3] = {0.0, 0.0, 0.0};
    int periodic[3] = {0, 0, 0};      // per axis, used when the Periodic policy is selected
    int iterations = 0;
    int iterationsMomentAvg = 0;      // average over the last iterationsMomentAvg steps
    int err_every_it = -1;
    int probe_every_it = -1;
    int probe_iterations = -1;
    int ProbeLocationLat[3] = {0, 0, 0};
    double err = 0.0;
    // storage of the populations on the GPU (lbm.h LBM_STORAGE_*), device, learned-closure model
    int32_t storage = LBM_STORAGE_F32;
    int32_t device = 0;
    int32_t mlp_interval = 1;
    const lbm_mlp_model* mlp = nullptr;
    // outlet sponge of OutletNeighbourEquilibriumOmega(RF) (LBMConstants.h:74-76; -1: none)
    double omegaDumpingLow = -1.0, omegaDumpingHigh = -1.0;
    // output as the reference's loop writes it (SolverTurbulentLES.h:225-263): results/variables.<k/plot>.vtk
    // every plot_every_it steps, results/variablesTimeAvg.vtk after the average, results/probeData.csv per
    // probe sample.  No files while results_dir is empty.
    int plot_every_it = -1;
    std::string results_dir;
    std::string InitFileName;         // InitializationEquilibriumVariables: the VTK file under results_dir
    double Crho = 1.0, Cpressure = 1.0, Cu = 1.0, Ct = 1.0;     // conversion factors (physical / lattice)
    double resolution_factor = 1.0, additional_factor = 0.5;   // VTK header geometry (geometry mesher)
    double BBmin[3] = {0.0, 0.0, 0.0};
    // physical inputs of NonDimensiolnaliseFactorsVelocity (LBMConstants.h:12-64); convertToLattice
    // converts when ny_fyz > 0, else the lattice-unit fields above are used as given
    double BBmax[3] = {0.0, 0.0, 0.0};
    double rho_fyz = 1.0, ny_fyz = 0.0, u_guess_fyz = 0.0, conversion_factor_fyz = 1.0, U_lb = 0.05;
    double L_fyz = 0.0, Cl = 1.0, Cm = 1.0, Cu_inverse = 1.0, Re = 0.0, omega = 0.0;  // set by the conversion
    // the reference sets tau = ny / 3 + 1/2 (NonDimensiolnaliseFactorsVelocity.h:66); nu = (tau - 1/2) / 3
    // gives 3 ny + 1/2, used unless tau_ref_compat
    bool tau_ref_compat = false;
    // initializeSimulationData (SolverTurbulentLES.h:276-323): step counts from physical times (-1: unset)
    double time = -1.0, plot_every = -1.0, err_every = -1.0;
    double ProbeLocation[3] = {0.0, 0.0, 0.0};
    // the preprocessor's inputs (preprocess.cpp:41-45): OFF file, output name, the point outside
    std::string file_name, mesh_name;
    double point_outside[3] = {-1.0, -1.0, -1.0};
};

struct LBMData {
    std::vector<int32_t> meshFluid;            // reference flag encoding, x fastest
    std::vector<lbm_bc_inlet> meshBoundaryInlet;
    std::vector<lbm_bc_outlet> meshBoundaryOutlet;
    std::vector<lbm_bc_symmetry> meshBoundarySymmetry;  // used with BounceSymmetryHalf
    std::vector<lbm_bc_periodic> meshBoundaryPeriodic;  // mesher output; the kernels wrap periodic axes by index
    std::vector<double> rhoInit, uInit;        // optional initial fields (else VelocityInit everywhere)
    std::vector<double> rho, u;                // host copies after the run (u: ux[N], uy[N], uz[N])
    std::vector<double> rhoTimeAvg, uTimeAvg, uuTimeAvg;
    std::vector<double> probe;                 // u_x, u_y, u_z, rho per probe sample
    std::vector<double> df;                    // populations [v][z][y][x] after readPopulations()
    std::vector<double> errors;                // ErrorQuadratic values, one per evaluation
};

class Error : public std::runtime_error {
public:
    Error(lbm_status s, const std::string& m) : std::runtime_error(m), status(s) {}
    lbm_status status;
};

// geometry/geometryObjectCuboid.h:9-52: the axis box spanned by three corners; id is the negative flag
// its cells get (-1 inlet, -2 outlet or symmetry, -3 periodic)
struct geometryObjectCuboid {
    lbm_cuboid c{};
    geometryObjectCuboid(const double X1[3], const double X2[3], const double X3[3], int id) {
        for (int a = 0; a < 3; a++) { c.x1[a] = X1[a]; c.x2[a] = X2[a]; c.x3[a] = X3[a]; }
        c.id = id;
    }
};

// geometry/geometryMesherBoundary.h: the wall pass and the cuboid boundary passes on Data.meshFluid (x
// fastest, changed in place) with the sampling frame of Constants (dimensions, resolution_factor,
// additional_factor, BBmin); the records go straight into Data's lists (the reference's
// compileBoundaryArray* copies, :486-603, are no-ops here).  Host code of the C ABI (lbm_mesher_*).
class geometryMesherBoundary {
public:
    geometryMesherBoundary(LBMConstants& constants, LBMData& data) : C(constants), D(data) {}

    void meshingBoundaryWall(bool /*verbose*/) {
        run(lbm_mesher_wall_pass(D.meshFluid.data(), C.dimX_int, C.dimY_int, C.dimZ_int));
    }
    void meshingBoundaryConditionInletUniform(const geometryObjectCuboid& cub, const float normal[3],
                                              const float velocity[3], bool /*verbose*/) {
        grow(D.meshBoundaryInlet, cub.c, [&](lbm_bc_inlet* r, int64_t cap, int64_t* n) {
            return lbm_mesher_inlet_uniform(&frame_, flags(), &cub.c, normal, velocity, r, cap, n);
        });
    }
    void meshingBoundaryConditionInletParaboloidCircle(const geometryObjectCuboid& cub, const double center[3],
                                                       float radius, const float normal[3], float mean_velocity,
                                                       bool /*verbose*/) {
        grow(D.meshBoundaryInlet, cub.c, [&](lbm_bc_inlet* r, int64_t cap, int64_t* n) {
            return lbm_mesher_inlet_paraboloid_circle(&frame_, flags(), &cub.c, center, radius, normal, mean_velocity,
                                                      r, cap, n);
        });
    }
    // the inlet dimensions along the normal are set to 1 on return, as the reference's by-reference arguments
    void meshingBoundaryConditionInletParaboloidRectangle(const geometryObjectCuboid& cub, const double center[3],
                                                          float& dimX, float& dimY, float& dimZ, const float normal[3],
                                                          float mean_velocity, bool /*verbose*/) {
        float d[3] = {dimX, dimY, dimZ};
        grow(D.meshBoundaryInlet, cub.c, [&](lbm_bc_inlet* r, int64_t cap, int64_t* n) {
            return lbm_mesher_inlet_paraboloid_rectangle(&frame_, flags(), &cub.c, center, d, normal, mean_velocity,
                                                         r, cap, n);
        });
        dimX = d[0]; dimY = d[1]; dimZ = d[2];
    }
    void meshingBoundaryConditionOutlet(const geometryObjectCuboid& cub, const float normal[3], float density,
                                        bool /*verbose*/) {
        grow(D.meshBoundaryOutlet, cub.c, [&](lbm_bc_outlet* r, int64_t cap, int64_t* n) {
            return lbm_mesher_outlet(&frame_, flags(), &cub.c, normal, density, r, cap, n);
        });
    }
    void meshingBoundaryConditionSymmetry(const geometryObjectCuboid& cub, const float normal[3], bool /*verbose*/) {
        grow(D.meshBoundarySymmetry, cub.c, [&](lbm_bc_symmetry* r, int64_t cap, int64_t* n) {
            return lbm_mesher_symmetry(&frame_, flags(), &cub.c, normal, r, cap, n);
        });
    }
    void meshingBoundaryConditionPeriodic(const geometryObjectCuboid& cub, const float normal[3], int periodicIndex,
                                          bool /*verbose*/) {
        grow(D.meshBoundaryPeriodic, cub.c, [&](lbm_bc_periodic* r, int64_t cap, int64_t* n) {
            return lbm_mesher_periodic(&frame_, flags(), &cub.c, normal, periodicIndex, r, cap, n);
        });
    }
    void compileBoundaryArrayInlets(bool) {}
    void compileBoundaryArrayOutlets(bool) {}
    void compileBoundaryArraySymmetry(bool) {}
    void compileBoundaryArrayPeriodic(bool) {}
    void compileBoundaryArrayWall(bool) {}  // wall links are found from the flags by the kernels
    void arrayTransfer(bool) {}             // initializeSimulation uploads flags and records

private:
    LBMConstants& C;
    LBMData& D;
    lbm_mesh_frame frame_{};

    int32_t* flags() {
        const size_t N = (size_t)C.dimX_int * C.dimY_int * C.dimZ_int;
        if (D.meshFluid.size() != N) throw Error(LBM_ERR_INVALID, "meshFluid has the wrong size");
        frame_.dims[0] = C.dimX_int; frame_.dims[1] = C.dimY_int; frame_.dims[2] = C.dimZ_int;
        frame_.resolution_factor = (float)C.resolution_factor;
        frame_.additional_factor = (float)C.additional_factor;
        for (int a = 0; a < 3; a++) frame_.bbmin[a] = (float)C.BBmin[a];
        return D.meshFluid.data();
    }
    static void run(lbm_status s) {
        if (s != LBM_OK) throw Error(s, std::string("mesher: ") + lbm_mesher_last_error());
    }
    // room for the cells of the cuboid's index box widened by one cell per side (centre test bound)
    int64_t bound(const lbm_cuboid& c) const {
        const int dims[3] = {C.dimX_int, C.dimY_int, C.dimZ_int};
        int64_t n = 1;
        for (int a = 0; a < 3; a++) {
            const double lo = std::fmin(c.x1[a], std::fmin(c.x2[a], c.x3[a]));
            const double hi = std::fmax(c.x1[a], std::fmax(c.x2[a], c.x3[a]));
            const double r = C.resolution_factor, ad = C.additional_factor, bb = C.BBmin[a];
            const double i0 = std::fmax(0.0, std::floor((lo - bb) * r + ad - 0.5) - 1);
            const double i1 = std::fmin(dims[a] - 1.0, std::ceil((hi - bb) * r + ad - 0.5) + 1);
            n *= i1 >= i0 ? (int64_t)(i1 - i0) + 1 : 0;
        }
        return n;
    }
    template <class Rec, class Pass>
    void grow(std::vector<Rec>& v, const lbm_cuboid& c, Pass pass) {
        const int64_t have = (int64_t)v.size();
        const int64_t cap = have + bound(c);
        v.resize((size_t)cap);
        int64_t n = have;
        const lbm_status s = pass(v.data(), cap, &n);
        v.resize((size_t)(s == LBM_OK ? n : have));
        run(s);
    }
};

// A lattice made periodic the reference's way (Periodic.h: per axis two planes of -3 nodes whose records
// point at each other) as the index-wrapped lattice the kernels run: with the pair at planes p < q of an
// axis, planes p .. q-1 are kept (plane q repeats plane p), the axis wraps (C.periodic), -3 flags become
// plain fluid and the inlet, outlet and symmetry records move with the planes (those on dropped planes
// are dropped).  D.meshBoundaryPeriodic is cleared.  The two forms step identically.
inline void foldPeriodic(LBMConstants& C, LBMData& D) {
    const int n[3] = {C.dimX_int, C.dimY_int, C.dimZ_int};
    int lo[3] = {0, 0, 0}, hi[3] = {n[0], n[1], n[2]};
    for (int a = 0; a < 3; a++) {
        int planes[2] = {-1, -1}, idx[2] = {-1, -1}, np_ = 0;
        for (const auto& r : D.meshBoundaryPeriodic) {
            int axis = -1, cnt = 0;
            for (int b = 0; b < 3; b++)
                if (r.normal[b] != 0) { axis = b; cnt++; }
            if (cnt != 1) throw Error(LBM_ERR_INVALID, "periodic record with a normal off the axes");
            if (axis != a) continue;
            const int pl = a == 0 ? r.vertex.x : a == 1 ? r.vertex.y : r.vertex.z;
            int e = 0;
            while (e < np_ && !(planes[e] == pl && idx[e] == r.periodic_index)) e++;
            if (e == np_) {
                if (np_ == 2) throw Error(LBM_ERR_INVALID, "more than two periodic planes on one axis");
                planes[np_] = pl; idx[np_] = r.periodic_index; np_++;
            }
        }
        if (np_ == 0) continue;
        if (np_ != 2) throw Error(LBM_ERR_INVALID, "a periodic plane without its partner");
        const int p = std::min(planes[0], planes[1]), q = std::max(planes[0], planes[1]);
        const int ip = planes[0] == p ? idx[0] : idx[1], iq = planes[0] == p ? idx[1] : idx[0];
        if (p == q || ip != q || iq != p) throw Error(LBM_ERR_INVALID, "periodic planes that do not point at each other");
        lo[a] = p; hi[a] = q; C.periodic[a] = 1;
    }
    const int m[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    std::vector<int32_t> f((size_t)m[0] * m[1] * m[2]);
    for (int k = 0; k < m[2]; k++)
        for (int j = 0; j < m[1]; j++)
            for (int i = 0; i < m[0]; i++) {
                const int32_t v = D.meshFluid[((size_t)(k + lo[2]) * n[1] + (j + lo[1])) * n[0] + (i + lo[0])];
                f[((size_t)k * m[1] + j) * m[0] + i] = v == -3 ? 1 : v;
            }
    auto move = [&](auto& recs) {
        size_t w = 0;
        for (size_t e = 0; e < recs.size(); e++) {
            auto r = recs[e];
            int v[3] = {r.vertex.x - lo[0], r.vertex.y - lo[1], r.vertex.z - lo[2]};
            if (v[0] < 0 || v[1] < 0 || v[2] < 0 || v[0] >= m[0] || v[1] >= m[1] || v[2] >= m[2]) continue;
            r.vertex.x = v[0]; r.vertex.y = v[1]; r.vertex.z = v[2];
            recs[w++] = r;
        }
        recs.resize(w);
    };
    move(D.meshBoundaryInlet);
    move(D.meshBoundaryOutlet);
    move(D.meshBoundarySymmetry);
    D.meshBoundaryPeriodic.clear();
    D.meshFluid.swap(f);
    C.dimX_int = m[0]; C.dimY_int = m[1]; C.dimZ_int = m[2];
}

// preprocess/src/geometry/geometryHandlerOFF.h and geometryMesherOFF.h: the preprocessor's calls
// (preprocess.cpp:60-72) over lbm_voxelize_off.  The handler reads the OFF/NOFF file and its bounding box
// (float, as LBMConstants keeps it); the mesher sizes the lattice, ceil((BBmax - BBmin) res + 2 add) per
// axis, and fills meshFluid with 1 inside the polyhedron, 0 outside (the GPU voxelizer: ray parity along
// +x, bit-exact with the reference's segment test on its golden file).
struct geometryHandlerOFF {
    std::string path;
    double bbox[6] = {0, 0, 0, 0, 0, 0};
    int32_t dims[3] = {0, 0, 0};
    void polyhedronFromFile(const LBMConstants& C, bool /*verbose*/) {
        path = C.file_name;
        const lbm_status s =
            lbm_voxelize_off(path.c_str(), C.resolution_factor, C.additional_factor, C.point_outside, nullptr, dims, bbox, 0);
        if (s != LBM_OK) throw Error(s, "cannot read the OFF file " + path);
    }
    void polyhedronBbox(bool /*verbose*/) {}  // the bounding box comes with the read
    void writeToConstants(LBMConstants& C) const {
        for (int a = 0; a < 3; a++) { C.BBmin[a] = bbox[a]; C.BBmax[a] = bbox[3 + a]; }
    }
};

class geometryMesherOFF {
public:
    geometryMesherOFF(LBMConstants& constants, LBMData& data) : C(constants), D(data) {}
    // geometryMesherOFF.h:45-79: lattice dimensions from the bounding box
    void initialization(bool /*verbose*/) {
        for (int a = 0; a < 3; a++) {
            const float ext = (float)C.BBmax[a] - (float)C.BBmin[a];
            const int n = (int)std::ceil(ext * (float)C.resolution_factor + 2 * (float)C.additional_factor);
            (a == 0 ? C.dimX_int : a == 1 ? C.dimY_int : C.dimZ_int) = n;
        }
        D.meshFluid.assign((size_t)C.dimX_int * C.dimY_int * C.dimZ_int, 0);
    }
    // :81-112: 1 inside, 0 outside at every cell centre
    void meshingPolyhedron(const geometryHandlerOFF& H, const double point_outside[3], bool /*verbose*/) {
        int32_t dims[3];
        double bbox[6];
        // the voxelizer's own dimensions first: it writes that many flags
        lbm_status s = lbm_voxelize_off(H.path.c_str(), C.resolution_factor, C.additional_factor, point_outside, nullptr,
                                        dims, bbox, C.device);
        if (s != LBM_OK) throw Error(s, "cannot read the OFF file " + H.path);
        if (dims[0] != C.dimX_int || dims[1] != C.dimY_int || dims[2] != C.dimZ_int)
            throw Error(LBM_ERR_INVALID, "the lattice does not match the polyhedron's bounding box");
        D.meshFluid.resize((size_t)dims[0] * dims[1] * dims[2]);
        s = lbm_voxelize_off(H.path.c_str(), C.resolution_factor, C.additional_factor, point_outside, D.meshFluid.data(),
                             dims, bbox, C.device);
        if (s != LBM_OK) throw Error(s, "lbm_voxelize_off failed on " + H.path);
    }

private:
    LBMConstants& C;
    LBMData& D;
};

// postprocesors/outputerVTK.h and outputerMesh.h: the reference's writer and reader names over the C ABI's
// host code.  Files go under <results_dir or "results">/ with the reference's names; the fields are the
// host copies in LBMData (rho, u after runSimulation; rhoTimeAvg, uTimeAvg after an average).
struct outputerVTK {
    static std::string dir(const LBMConstants& C) { return C.results_dir.empty() ? std::string("results") : C.results_dir; }
    // one structured-points file with rho, p or pressure (rho cs2) and U, each times its factor
    static void variables(const std::string& path, const LBMConstants& C, const std::vector<double>& rho,
                          const std::vector<double>& u, const char* pname, double crho, double cp, double cu) {
        const size_t N = (size_t)C.dimX_int * C.dimY_int * C.dimZ_int;
        if (rho.size() != N || u.size() != 3 * N) throw Error(LBM_ERR_INVALID, "outputerVTK: fields not read back");
        std::vector<double> p(N);
        for (size_t i = 0; i < N; i++) p[i] = rho[i] / 3.0;
        const lbm_vtk_field f[3] = {{"rho", 1, rho.data(), crho}, {pname, 1, p.data(), cp}, {"U", 3, u.data(), cu}};
        write(path, "LBE variables", C, f, 3);
    }
    static void write(const std::string& path, const char* title, const LBMConstants& C, const lbm_vtk_field* f,
                      int n) {
        const int32_t dims[3] = {C.dimX_int, C.dimY_int, C.dimZ_int};
        const lbm_status st = lbm_vtk_write(path.c_str(), title, dims, C.resolution_factor, C.additional_factor,
                                            C.BBmin, f, n);
        if (st != LBM_OK) throw Error(st, std::string("lbm_vtk_write: ") + lbm_vtk_last_error());
    }
    // :26-56: the flag field as "object", title "LBE <filename>"
    static void MeshVTK(const LBMData& D, const LBMConstants& C, const std::string& filename) {
        std::vector<double> fl(D.meshFluid.begin(), D.meshFluid.end());
        const lbm_vtk_field f = {"object", 1, fl.data(), 1.0};
        write(dir(C) + "/" + filename + ".vtk", ("LBE " + filename).c_str(), C, &f, 1);
    }
    // :59-187 (physical units, results/variables.<step>.vtk) and :189-316 (lattice, variablesLattice<step>.vtk)
    static void variablesVTK(const LBMData& D, const LBMConstants& C, int step, bool /*verbose*/) {
        variables(dir(C) + "/variables." + std::to_string(step) + ".vtk", C, D.rho, D.u, "p", C.Crho, C.Cpressure,
                  C.Cu);
    }
    static void variablesLatticeVTK(const LBMData& D, const LBMConstants& C, int step, bool /*verbose*/) {
        variables(dir(C) + "/variablesLattice" + std::to_string(step) + ".vtk", C, D.rho, D.u, "pressure", 1, 1, 1);
    }
    // :318-447 and :449-576 (both write results/variablesTimeAvg.vtk)
    static void variablesTimeAvgVTK(const LBMData& D, const LBMConstants& C, bool /*verbose*/) {
        variables(dir(C) + "/variablesTimeAvg.vtk", C, D.rhoTimeAvg, D.uTimeAvg, "pressure", C.Crho, C.Cpressure, C.Cu);
    }
    static void variablesTimeAvgLatticeVTK(const LBMData& D, const LBMConstants& C, bool /*verbose*/) {
        variables(dir(C) + "/variablesTimeAvg.vtk", C, D.rhoTimeAvg, D.uTimeAvg, "pressure", 1, 1, 1);
    }
    // :660-740: one population (reference velocity order) from D.df as "DFunciton_<velocity>", as the
    // reference names the field (:690), in results/distributionFunction<velocity>.vtk
    static void distributionFunctionVTK(const LBMData& D, const LBMConstants& C, int velocity, bool /*verbose*/) {
        const size_t N = (size_t)C.dimX_int * C.dimY_int * C.dimZ_int;
        if (velocity < 0 || velocity > 26 || D.df.size() != 27 * N)
            throw Error(LBM_ERR_INVALID, "distributionFunctionVTK: velocity out of range or populations not read back");
        const std::string name = "DFunciton_" + std::to_string(velocity);
        const lbm_vtk_field f = {name.c_str(), 1, D.df.data() + (size_t)velocity * N, 1.0};
        write(dir(C) + "/distributionFunction" + std::to_string(velocity) + ".vtk", "LBE variables", C, &f, 1);
    }
    // :824-851: one probe line appended to results/probeData.csv
    static void probeWriteOut(const LBMConstants& C, double velX, double velY, double velZ, double rho) {
        const double s[4] = {velX, velY, velZ, rho};
        const std::string path = dir(C) + "/probeData.csv";
        const lbm_status st = lbm_probe_csv_append(path.c_str(), C.Ct * C.probe_every_it, s, C.Cu, C.Crho, C.Cpressure);
        if (st != LBM_OK) throw Error(st, std::string("lbm_probe_csv_append: ") + lbm_vtk_last_error());
    }
};

struct outputerMesh {
    // outputerMesh.h:19-56: results/<filename>.txt from meshFluid and the header constants
    static void MeshMatrixOut(const LBMData& D, const LBMConstants& C, const std::string& filename) {
        const int32_t dims[3] = {C.dimX_int, C.dimY_int, C.dimZ_int};
        const double bbox[6] = {C.BBmin[0], C.BBmin[1], C.BBmin[2], C.BBmax[0], C.BBmax[1], C.BBmax[2]};
        const std::string path = outputerVTK::dir(C) + "/" + filename + ".txt";
        const lbm_status st =
            lbm_mesh_matrix_write(path.c_str(), D.meshFluid.data(), dims, C.resolution_factor, C.additional_factor, bbox);
        if (st != LBM_OK) throw Error(st, std::string("lbm_mesh_matrix_write: ") + lbm_mesh_matrix_last_error());
    }
    // :59-211: dimensions, resolution_factor, additional_factor, BBmin / BBmax and meshFluid from the file
    static void MeshMatrixIn(LBMData& D, LBMConstants& C, const std::string& filename, bool verbose) {
        const std::string path = outputerVTK::dir(C) + "/" + filename + ".txt";
        int32_t dims[3];
        double res = 0, add = 0, bbox[6];
        lbm_status st = lbm_mesh_matrix_read(path.c_str(), nullptr, 0, dims, &res, &add, bbox);
        if (st != LBM_OK) throw Error(st, std::string("lbm_mesh_matrix_read: ") + lbm_mesh_matrix_last_error());
        D.meshFluid.resize((size_t)dims[0] * dims[1] * dims[2]);
        st = lbm_mesh_matrix_read(path.c_str(), D.meshFluid.data(), (int64_t)D.meshFluid.size(), dims, nullptr, nullptr,
                                  nullptr);
        if (st != LBM_OK) throw Error(st, std::string("lbm_mesh_matrix_read: ") + lbm_mesh_matrix_last_error());
        C.dimX_int = dims[0]; C.dimY_int = dims[1]; C.dimZ_int = dims[2];
        C.resolution_factor = res; C.additional_factor = add;
        for (int a = 0; a < 3; a++) { C.BBmin[a] = bbox[a]; C.BBmax[a] = bbox[3 + a]; }
        if (verbose) std::printf("Mesh %s read: %d x %d x %d\n", path.c_str(), dims[0], dims[1], dims[2]);
    }
};

// nonDimensionalisions/NonDimensiolnaliseFactorsVelocity.h: lattice units from the physical inputs, in
// the reference's float arithmetic (RealType = float, LBMTraits.h:72)
struct NonDimensiolnaliseFactorsVelocity {
    // :20-85.  Cl = L_x / nx with L_x = |BBmax_x - BBmin_x| * conversion_factor_fyz; Cu = u_guess / U_lb;
    // Ct = Cl / Cu; Crho = rho_fyz; Cm = Crho Cl^3; Cpressure = Cm / Cl / Ct^2; Re = u_guess L_x / nu_fyz;
    // ny = nu_fyz Ct / Cl^2; tau, omega = 1 / tau.  The reference asserts U_lb < cs and 0.5 < tau < 0.99
    // (:29, :81): both raise here.
    static void nonDimensionalize(LBMConstants& C) {
        using R = float;
        const R cs = 1.f / std::sqrt(3.f);
        if (!((R)C.U_lb < cs)) throw Error(LBM_ERR_INVALID, "U_lb must be below the speed of sound");
        const R L = std::fabs((R)C.BBmax[0] - (R)C.BBmin[0]) * (R)C.conversion_factor_fyz;
        const R Cl = L / (R)C.dimX_int;
        const R Cu = (R)C.u_guess_fyz / (R)C.U_lb;
        const R Ct = Cl / Cu;
        const R Crho = (R)C.rho_fyz;
        const R Cm = Crho * Cl * Cl * Cl;
        const R ny = (R)C.ny_fyz * Ct / Cl / Cl;
        const R tau = C.tau_ref_compat ? ny / 3.f + 0.5f : 3.f * ny + 0.5f;
        if (!(tau > 0.5f && tau < 0.99f))
            throw Error(LBM_ERR_INVALID, "tau = " + std::to_string(tau) + " outside (0.5, 0.99): change the "
                                         "resolution or the lattice speed");
        C.L_fyz = L; C.Cl = Cl; C.Cu = Cu; C.Cu_inverse = (R)1 / Cu; C.Ct = Ct; C.Crho = Crho; C.Cm = Cm;
        C.Cpressure = Cm / Cl / Ct / Ct;
        C.Re = (R)C.u_guess_fyz * L / (R)C.ny_fyz;
        C.ny = ny; C.tau = tau; C.omega = 1.f / tau;
    }
    // :87-108: inlet velocities times Cu_inverse
    static void nonDimensionalizeInlet(std::vector<lbm_bc_inlet>& in, const LBMConstants& C) {
        for (auto& r : in)
            for (int a = 0; a < 3; a++) r.velocity[a] = (float)((float)r.velocity[a] * (float)C.Cu_inverse);
    }
    // :110-130: outlet densities / Cm * Cl^3
    static void nonDimensionalizeOutlet(std::vector<lbm_bc_outlet>& out, const LBMConstants& C) {
        const float Cm = (float)C.Cm, Cl = (float)C.Cl;
        for (auto& r : out) r.density = (float)r.density / Cm * Cl * Cl * Cl;
    }
};

inline void check(lbm_status s, const lbm_ctx* ctx, const char* what) {
    if (s != LBM_OK) throw Error(s, std::string(what) + ": " + lbm_last_error(ctx));
}

template <typename MODELTYPE, typename INITIALIZATIONTYPE, typename COLLISIONTYPE, typename STREAMINGTYPE,
          typename BOUNCEBACKWALLTYPE, typename SYMMETRYTYPE, typename PERIODICTYPE, typename INLETTYPE,
          typename OUTLETTYPE, typename MOMENTTYPE, typename TURBULENCETYPE, typename ERRORTYPE, typename NONDYM,
          typename MOMENTTIMEAVGTYPE>
class SolverTurbulentLES {
    static_assert(MODELTYPE::numberOfDiscreteVelocities == 27, "the kernels are D3Q27");
    static_assert(std::is_same<STREAMINGTYPE, StreamingAB>::value, "streaming: StreamingAB (AA pattern in place)");
    static_assert(std::is_same<BOUNCEBACKWALLTYPE, BounceBackWallHalf>::value ||
                      std::is_same<BOUNCEBACKWALLTYPE, BounceBackWallHalfMesh>::value,
                  "wall: BounceBackWallHalf or BounceBackWallHalfMesh");
    static_assert(std::is_same<SYMMETRYTYPE, NoSymmetry>::value || std::is_same<SYMMETRYTYPE, BounceSymmetryHalf>::value,
                  "symmetry: NoSymmetry or BounceSymmetryHalf");
    static_assert(std::is_same<OUTLETTYPE, OutletDensityInterpolated>::value ||
                      std::is_same<OUTLETTYPE, OutletNeighbourEquilibrium>::value ||
                      std::is_same<OUTLETTYPE, OutletNeighbourEquilibriumOmega>::value ||
                      std::is_same<OUTLETTYPE, OutletNeighbourEquilibriumOmegaRF>::value ||
                      std::is_same<OUTLETTYPE, OutletDensityEquilibrium>::value,
                  "outlet: OutletDensityInterpolated, OutletNeighbourEquilibrium(Omega, OmegaRF) or "
                  "OutletDensityEquilibrium");
    static_assert(std::is_same<MOMENTTYPE, MomentDensityVelocityN27>::value, "moments: MomentDensityVelocityN27");
    static_assert(std::is_same<ERRORTYPE, ErrorQuadratic>::value, "error: ErrorQuadratic");
    static_assert(std::is_same<INITIALIZATIONTYPE, InitializationEquilibriumConstVector>::value ||
                      std::is_same<INITIALIZATIONTYPE, InitializationEquilibriumVariables>::value,
                  "initialisation: InitializationEquilibriumConstVector or InitializationEquilibriumVariables");
    static_assert(std::is_same<MOMENTTIMEAVGTYPE, MomentTimeAvg>::value, "time average: MomentTimeAvg");

public:
    SolverTurbulentLES() = delete;
    SolverTurbulentLES(LBMConstants& constants, LBMData& data) : Constants(constants), Data(data) {}
    SolverTurbulentLES(const SolverTurbulentLES&) = delete;
    SolverTurbulentLES& operator=(const SolverTurbulentLES&) = delete;
    ~SolverTurbulentLES() {
        if (ctx) lbm_destroy(ctx);
    }

    // SolverTurbulentLES.h:270-274: NONDYM::nonDimensionalize when physical inputs are given (ny_fyz > 0);
    // with lattice-unit constants (ny_fyz = 0) nothing changes.  After a conversion, initializeSimulation
    // also converts the inlet velocities and outlet densities (SolverTurbulentLES.h:118, :124) and the
    // initial state (rho_fyz / Cm Cl^3, VelocityInit / Cu: InitializationEquilibriumConstVector.h:79-82).
    void convertToLattice(bool verbose) {
        if (!(Constants.ny_fyz > 0)) return;
        NONDYM::nonDimensionalize(Constants);
        converted = true;
        if (verbose)
            std::printf("Cl %g Cu %g Ct %g Re %g ny %g tau %g\n", Constants.Cl, Constants.Cu, Constants.Ct,
                        Constants.Re, Constants.ny, Constants.tau);
    }

    // SolverTurbulentLES.h:276-323: step counts from physical times (plot_every, err_every, time over Ct)
    // and the probe position in lattice cells (round(x / (BBmax - BBmin + 2 additional / resolution) n)).
    // One of plot_every / plot_every_it and of err_every / err_every_it must be given, as the reference
    // asserts.  The reference's probe asserts test lat >= dim (:313-315), the reverse of their message; the
    // probe must lie inside the lattice here.
    void initializeSimulationData(bool verbose) {
        using R = float;
        auto steps = [&](int& it, double every, const char* what) {
            if (it == -1 && every != -1) it = (int)std::ceil((R)every / (R)Constants.Ct);
            else if (it == -1) throw Error(LBM_ERR_INVALID, std::string("give ") + what + " or " + what + "_it");
        };
        steps(Constants.plot_every_it, Constants.plot_every, "plot_every");
        steps(Constants.err_every_it, Constants.err_every, "err_every");
        if (Constants.time >= 0) Constants.iterations = (int)std::ceil((R)Constants.time / (R)Constants.Ct);
        if (verbose) std::printf("Plotting every %d iterations; %d iterations.\n", Constants.plot_every_it,
                                 Constants.iterations);
        if (Constants.probe_every_it != -1) {
            const int dims[3] = {Constants.dimX_int, Constants.dimY_int, Constants.dimZ_int};
            const R pad = 2 * ((R)Constants.additional_factor / (R)Constants.resolution_factor);
            for (int a = 0; a < 3; a++) {
                const R ext = (R)Constants.BBmax[a] - (R)Constants.BBmin[a] + pad;
                const int lat = (int)std::round((R)Constants.ProbeLocation[a] / ext * (R)dims[a]);
                if (lat < 0 || lat >= dims[a]) throw Error(LBM_ERR_INVALID, "Probe must be in the domain!");
                Constants.ProbeLocationLat[a] = lat;
            }
        }
    }

    // the context, geometry, boundary records and the equilibrium initial state
    // (SolverTurbulentLES.h:103-146; InitializationEquilibriumConstVector.h:20-141)
    void initializeSimulation(bool verbose) {
        lbm_config c{};
        c.nx = Constants.dimX_int; c.ny = Constants.dimY_int; c.nz = Constants.dimZ_int;
        for (int a = 0; a < 3; a++) c.periodic[a] = PERIODICTYPE::on && !laminar_loop ? Constants.periodic[a] : 0;
        c.collision = COLLISIONTYPE::code;
        c.closure = COLLISIONTYPE::laminar ? LBM_CLOSURE_NONE : TURBULENCETYPE::code;
        c.storage = Constants.storage;
        c.inlet_kind = INLETTYPE::code;
        c.nu = Constants.ny;
        c.tau = Constants.tau;
        c.cles = Constants.CLES;
        c.force[0] = Constants.Fx; c.force[1] = Constants.Fy; c.force[2] = Constants.Fz;
        c.rho0 = Constants.rho0;
        c.f16_scale_log2 = 10;
        c.device = Constants.device;
        c.mlp_interval = Constants.mlp_interval;
        c.outlet_kind = OUTLETTYPE::code;
        c.omega_dumping_low = COLLISIONTYPE::laminar ? 0.0 : Constants.omegaDumpingLow;    // a sponge of slope 0
        c.omega_dumping_high = COLLISIONTYPE::laminar ? 0.0 : Constants.omegaDumpingHigh;
        if (ctx) lbm_destroy(ctx);
        ctx = nullptr;
        check(lbm_create(&c, &ctx), nullptr, "lbm_create");
        const size_t N = (size_t)c.nx * c.ny * c.nz;
        if (Data.meshFluid.size() != N) throw Error(LBM_ERR_INVALID, "meshFluid has the wrong size");
        check(lbm_set_flags(ctx, Data.meshFluid.data()), ctx, "lbm_set_flags");
        std::vector<lbm_bc_inlet> inlets = Data.meshBoundaryInlet;
        std::vector<lbm_bc_outlet> outlets = Data.meshBoundaryOutlet;
        double rho_init = Constants.rho0, u_init[3] = {Constants.VelocityInit[0], Constants.VelocityInit[1],
                                                       Constants.VelocityInit[2]};
        if (converted) {
            NONDYM::nonDimensionalizeInlet(inlets, Constants);
            NONDYM::nonDimensionalizeOutlet(outlets, Constants);
            const float Cl = (float)Constants.Cl;
            rho_init = (float)Constants.rho_fyz / (float)Constants.Cm * Cl * Cl * Cl;
            for (int a = 0; a < 3; a++) u_init[a] = (float)Constants.VelocityInit[a] * (float)Constants.Cu_inverse;
        }
        check(lbm_set_bc(ctx, inlets.data(), (int32_t)inlets.size(), outlets.data(), (int32_t)outlets.size()), ctx,
              "lbm_set_bc");
        if (SYMMETRYTYPE::on)
            check(lbm_set_symmetry(ctx, Data.meshBoundarySymmetry.data(), (int32_t)Data.meshBoundarySymmetry.size()),
                  ctx, "lbm_set_symmetry");
        if (std::is_same<INITIALIZATIONTYPE, InitializationEquilibriumVariables>::value) {
            const std::string path =
                (Constants.results_dir.empty() ? std::string("results") : Constants.results_dir) + "/" +
                Constants.InitFileName;
            std::vector<double> rho(N), u(3 * N);
            const int32_t dims[3] = {c.nx, c.ny, c.nz};
            const lbm_status s = lbm_vtk_read_variables(path.c_str(), dims, rho.data(), u.data());
            if (s != LBM_OK) throw Error(s, std::string("lbm_vtk_read_variables: ") + lbm_vtk_last_error());
            check(lbm_init_fields(ctx, rho.data(), u.data()), ctx, "lbm_init_fields");
        } else if (!Data.rhoInit.empty()) {
            if (Data.rhoInit.size() != N || Data.uInit.size() != 3 * N)
                throw Error(LBM_ERR_INVALID, "rhoInit / uInit have the wrong size");
            check(lbm_init_fields(ctx, Data.rhoInit.data(), Data.uInit.data()), ctx, "lbm_init_fields");
        } else {
            check(lbm_init_equilibrium(ctx, rho_init, u_init), ctx, "lbm_init_equilibrium");
        }
        if (std::is_same<TURBULENCETYPE, OmegaMLP>::value && !COLLISIONTYPE::laminar) {
            if (!Constants.mlp) throw Error(LBM_ERR_STATE, "OmegaMLP needs LBMConstants::mlp");
            check(lbm_mlp_load(ctx, Constants.mlp), ctx, "lbm_mlp_load");
        }
        if (verbose) std::printf("Initialization of simulation done (%d x %d x %d).\n", c.nx, c.ny, c.nz);
    }

    // u_x, u_y, u_z, rho of the probe cell appended to Data.probe (SolverTurbulentLES.h:150-177)
    void probeWrite() {
        double out[4];
        check(lbm_probe(ctx, Constants.ProbeLocationLat[0], Constants.ProbeLocationLat[1],
                        Constants.ProbeLocationLat[2], out),
              ctx, "lbm_probe");
        Data.probe.insert(Data.probe.end(), out, out + 4);
        if (!Constants.results_dir.empty()) {
            const std::string path = Constants.results_dir + "/probeData.csv";
            const lbm_status st = lbm_probe_csv_append(path.c_str(), Constants.Ct * Constants.probe_every_it, out,
                                                       Constants.Cu, Constants.Crho, Constants.Cpressure);
            if (st != LBM_OK) throw Error(st, std::string("lbm_probe_csv_append: ") + lbm_vtk_last_error());
        }
    }

    // outputerVTK::variablesVTK / variablesTimeAvgVTK (outputerVTK.h:59-187, :318-447): rho Crho,
    // p Cpressure (p = rho cs2) and U Cu, structured points
    // pressure_name: the field is "pressure" (time averages, lattice dumps), else "p"; lattice: factors 1
    void writeVTK(const std::string& path, const std::vector<double>& rho, const std::vector<double>& u,
                  bool pressure_name, bool lattice = false) {
        std::vector<double> p(rho.size());
        for (size_t i = 0; i < rho.size(); i++) p[i] = rho[i] / 3.0;
        const lbm_vtk_field f[3] = {{"rho", 1, rho.data(), lattice ? 1.0 : Constants.Crho},
                                    {pressure_name ? "pressure" : "p", 1, p.data(), lattice ? 1.0 : Constants.Cpressure},
                                    {"U", 3, u.data(), lattice ? 1.0 : Constants.Cu}};
        const int32_t dims[3] = {Constants.dimX_int, Constants.dimY_int, Constants.dimZ_int};
        const lbm_status st = lbm_vtk_write(path.c_str(), "LBE variables", dims, Constants.resolution_factor,
                                            Constants.additional_factor, Constants.BBmin, f, 3);
        if (st != LBM_OK) throw Error(st, std::string("lbm_vtk_write: ") + lbm_vtk_last_error());
    }

    // the reference's step loop (SolverTurbulentLES.h:179-268).  After step k: the state is added to the
    // time average when k > iterations - iterationsMomentAvg, the probe is sampled when
    // k % probe_every_it == 0 within the last probe_iterations steps, the error is evaluated when
    // k % err_every_it == 0 (k > 0) and a NaN error ends the loop.  The steps between two such events
    // go to the GPU as one lbm_step call.
    void runSimulation() {
        if (!ctx) throw Error(LBM_ERR_STATE, "runSimulation before initializeSimulation");
        const int it = Constants.iterations;
        const int avg = Constants.iterationsMomentAvg;
        const int avg_begin = it - avg + 1;  // lbm_timeavg counts the states produced after the call
        auto probe_after = [&](int k) {
            return !laminar_loop && Constants.probe_every_it > 0 && k % Constants.probe_every_it == 0 &&
                   k >= it - Constants.probe_iterations;
        };
        auto err_after = [&](int k) { return Constants.err_every_it > 0 && k % Constants.err_every_it == 0 && k != 0; };
        auto plot_after = [&](int k) {
            return !Constants.results_dir.empty() && Constants.plot_every_it > 0 && k % Constants.plot_every_it == 0 &&
                   (k != 0 || laminar_loop);
        };
        const size_t N = (size_t)Constants.dimX_int * Constants.dimY_int * Constants.dimZ_int;
        bool averaging = false;
        int k = 0;  // steps done
        while (k < it) {
            if (avg > 0 && !averaging && k >= avg_begin) {
                check(lbm_timeavg_begin(ctx), ctx, "lbm_timeavg_begin");
                averaging = true;
            }
            int j = k;  // the last step of this batch: the first with an event after it
            while (j < it - 1 && !probe_after(j) && !err_after(j) && !plot_after(j) &&
                   !(avg > 0 && !averaging && j + 1 >= avg_begin))
                j++;
            check(lbm_step(ctx, j - k + 1), ctx, "lbm_step");
            k = j + 1;
            if (probe_after(j)) probeWrite();
            if (err_after(j)) {
                double e = 0.0;
                check(lbm_error_evaluation(ctx, &e), ctx, "lbm_error_evaluation");
                Constants.err = e;
                Data.errors.push_back(e);
                if (std::isnan(e)) break;
            }
            if (plot_after(j)) {
                Data.rho.resize(N);
                Data.u.resize(3 * N);
                check(lbm_get_moments(ctx, Data.rho.data(), Data.u.data()), ctx, "lbm_get_moments");
                if (laminar_loop)  // outputerVTK::variablesLatticeVTK (outputerVTK.h:189-316): lattice units
                    writeVTK(Constants.results_dir + "/variablesLattice" + std::to_string(j / Constants.plot_every_it) +
                                 ".vtk",
                             Data.rho, Data.u, true, true);
                else
                    writeVTK(Constants.results_dir + "/variables." + std::to_string(j / Constants.plot_every_it) +
                                 ".vtk",
                             Data.rho, Data.u, false);
            }
        }
        if (averaging) check(lbm_timeavg_end(ctx), ctx, "lbm_timeavg_end");
        check(lbm_synchronize(ctx), ctx, "lbm_synchronize");
        Data.rho.resize(N);
        Data.u.resize(3 * N);
        check(lbm_get_moments(ctx, Data.rho.data(), Data.u.data()), ctx, "lbm_get_moments");
        if (averaging) {
            Data.rhoTimeAvg.resize(N);
            Data.uTimeAvg.resize(3 * N);
            Data.uuTimeAvg.resize(6 * N);
            check(lbm_timeavg_get(ctx, Data.rhoTimeAvg.data(), Data.uTimeAvg.data(), Data.uuTimeAvg.data(), nullptr),
                  ctx, "lbm_timeavg_get");
            if (!Constants.results_dir.empty())
                writeVTK(Constants.results_dir + "/variablesTimeAvg.vtk", Data.rhoTimeAvg, Data.uTimeAvg, true);
        }
    }

    lbm_ctx* context() { return ctx; }

    // the populations in the reference layout into Data.df (for distributionFunctionVTK)
    void readPopulations() {
        if (!ctx) throw Error(LBM_ERR_STATE, "readPopulations before initializeSimulation");
        Data.df.resize((size_t)27 * Constants.dimX_int * Constants.dimY_int * Constants.dimZ_int);
        check(lbm_get_populations(ctx, Data.df.data()), ctx, "lbm_get_populations");
    }

    LBMConstants& Constants;
    LBMData& Data;

protected:
    // SolverLaminar's loop (SolverLaminar.h:127-204): no probe, a lattice-unit dump also after the first
    // step, and no periodic hook (the reference's laminar loop never calls PERIODICTYPE)
    bool laminar_loop = false;

private:
    lbm_ctx* ctx = nullptr;
    bool converted = false;  // convertToLattice converted physical inputs
};

// solvers/SolverLaminar.h:61-237: the same policies without a turbulence model.  The step runs with the
// global omega = 1/tau (OmegaNo); initializeSimulation first runs initializeSimulationData, as the
// reference's does (:99).
template <typename MODELTYPE, typename INITIALIZATIONTYPE, typename COLLISIONTYPE, typename STREAMINGTYPE,
          typename BOUNCEBACKWALLTYPE, typename SYMMETRYTYPE, typename PERIODICTYPE, typename INLETTYPE,
          typename OUTLETTYPE, typename MOMENTTYPE, typename ERRORTYPE, typename NONDYM, typename MOMENTTIMEAVGTYPE>
class SolverLaminar
    : public SolverTurbulentLES<MODELTYPE, INITIALIZATIONTYPE, COLLISIONTYPE, STREAMINGTYPE, BOUNCEBACKWALLTYPE,
                                SYMMETRYTYPE, PERIODICTYPE, INLETTYPE, OUTLETTYPE, MOMENTTYPE, OmegaNo, ERRORTYPE, NONDYM,
                                MOMENTTIMEAVGTYPE> {
    using Base = SolverTurbulentLES<MODELTYPE, INITIALIZATIONTYPE, COLLISIONTYPE, STREAMINGTYPE, BOUNCEBACKWALLTYPE,
                                    SYMMETRYTYPE, PERIODICTYPE, INLETTYPE, OUTLETTYPE, MOMENTTYPE, OmegaNo, ERRORTYPE,
                                    NONDYM, MOMENTTIMEAVGTYPE>;

public:
    SolverLaminar(LBMConstants& constants, LBMData& data) : Base(constants, data) { this->laminar_loop = true; }
    void initializeSimulation(bool verbose) {
        this->initializeSimulationData(verbose);
        Base::initializeSimulation(verbose);
    }
};

}  // namespace lbm_gb300
