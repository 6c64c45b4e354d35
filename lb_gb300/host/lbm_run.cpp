// lbm_run.cpp - C++ host driver: builds a case, runs it through SolverTurbulentLES (include/lbm_solver.hpp)
// on the GPU and writes profiles and timings.  The counterpart of the reference's 3D/simulation/main.cu,
// which sets LBMConstants, meshes the geometry and calls initializeSimulation / runSimulation.
//
//   lbm_run cavity  [--n 64] [--steps 10000] [--re 1000] [--ulid 0.05] [--storage f64|f32|f16dev] [--out DIR]
//                   [--plot K]  (both cases: DIR/variables.<i>.vtk every K steps, DIR/variablesTimeAvg.vtk after
//                                the average, in lattice units, as the reference's outputerVTK writes them)
//   lbm_run channel [--nx 256 --ny 130 --nz 128] [--steps 20000] [--avg 5000] [--storage ...]
//                   [--re-tau 180] [--umax 0.05] [--amp 0.05] [--mlp model.bin] [--mlp-interval 1] [--out DIR]
//
// cavity (lid-driven, cumulant, no closure): writes DIR/centerline_ux_y.txt (u_x along y at x = z = n/2) and
// DIR/centerline_uy_x.txt.  channel (cumulant + Smagorinsky, or the learned closure with --mlp): periodic
// x and z, solid rows y = 0 and y = ny-1, body force for Re_tau; initial laminar profile plus seeded
// uniform noise (the splitmix64 generator of lb_gb300/cases.py); writes DIR/mean_profile.txt
// (y, <u_x>, <u_x'u_x'>, <u_y'u_y'>, <u_z'u_z'>, <u_x'u_y'> averaged over x, z and the last --avg steps).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "lbm_solver.hpp"

using namespace lbm_gb300;

namespace {

uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// U[0,1) per (seed, index, component), as lb_gb300.cases.uniform
double uniform01(uint64_t seed, uint64_t index, uint64_t component) {
    const uint64_t key = seed * 0x100000001B3ull + index * 8ull + component;
    return (double)(splitmix64(splitmix64(key)) >> 11) * (1.0 / 9007199254740992.0);
}

int32_t storage_of(const std::string& s) {
    if (s == "f64") return LBM_STORAGE_F64;
    if (s == "f32") return LBM_STORAGE_F32;
    if (s == "f16dev") return LBM_STORAGE_F16DEV;
    throw Error(LBM_ERR_INVALID, "storage must be f64, f32 or f16dev");
}

struct Args {
    std::map<std::string, std::string> kv;
    std::string get(const std::string& k, const std::string& d) const {
        auto it = kv.find(k);
        return it == kv.end() ? d : it->second;
    }
    double num(const std::string& k, double d) const { return std::atof(get(k, std::to_string(d)).c_str()); }
    int inum(const std::string& k, int d) const { return std::atoi(get(k, std::to_string(d)).c_str()); }
};

void write_columns(const std::string& path, const std::vector<std::vector<double>>& cols, const char* header) {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) throw Error(LBM_ERR_IO, "cannot write " + path);
    std::fprintf(f, "# %s\n", header);
    for (size_t i = 0; i < cols[0].size(); i++) {
        for (size_t c = 0; c < cols.size(); c++) std::fprintf(f, c ? " %.17g" : "%.17g", cols[c][i]);
        std::fprintf(f, "\n");
    }
    std::fclose(f);
}

template <class Solver>
double timed_run(Solver& s) {
    const auto t0 = std::chrono::steady_clock::now();
    s.runSimulation();
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

int run_cavity(const Args& a) {
    const int n = a.inum("n", 64);
    const double ulid = a.num("ulid", 0.05), re = a.num("re", 1000.0);
    LBMConstants C;
    LBMData D;
    C.dimX_int = C.dimY_int = C.dimZ_int = n;
    C.ny = ulid * n / re;
    C.iterations = a.inum("steps", 10000);
    C.storage = storage_of(a.get("storage", "f64"));
    C.err_every_it = a.inum("err-every", 1000);
    C.plot_every_it = a.inum("plot", -1);
    if (C.plot_every_it > 0) C.results_dir = a.get("out", ".");
    const size_t N = (size_t)n * n * n;
    D.meshFluid.assign(N, 1);
    auto at = [&](int i, int j, int k) -> int32_t& { return D.meshFluid[(size_t)i + (size_t)n * ((size_t)j + (size_t)n * k)]; };
    for (int k = 0; k < n; k++)
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++)
                if (i == 0 || i == n - 1 || j == 0 || k == 0 || k == n - 1) at(i, j, k) = 0;
    for (int k = 1; k < n - 1; k++)
        for (int i = 1; i < n - 1; i++) {
            at(i, n - 1, k) = -1;
            lbm_bc_inlet r{};
            r.vertex = {i, n - 1, k};
            r.normal[1] = 1.0f;
            r.velocity[0] = (float)ulid;
            r.regular = 1;
            D.meshBoundaryInlet.push_back(r);
        }
    check(lbm_mesher_wall_pass(D.meshFluid.data(), n, n, n), nullptr, "lbm_mesher_wall_pass");
    SolverTurbulentLES<D3Q27, InitializationEquilibriumConstVector, CollisionCumD3Q27Turbulent2015, StreamingAB,
                       BounceBackWallHalf, NoSymmetry, NoPeriodic, InletVelocityMovingWall, OutletDensityInterpolated,
                       MomentDensityVelocityN27, OmegaNo, ErrorQuadratic, NonDimensiolnaliseFactorsVelocity,
                       MomentTimeAvg>
        s(C, D);
    s.convertToLattice(true);
    s.initializeSimulation(true);
    const double sec = timed_run(s);
    const std::string out = a.get("out", ".");
    const int c = n / 2;
    std::vector<double> y, uxy, x, uyx;
    for (int j = 0; j < n; j++) {
        y.push_back(j);
        uxy.push_back(D.u[(size_t)c + (size_t)n * ((size_t)j + (size_t)n * c)] / ulid);
    }
    for (int i = 0; i < n; i++) {
        x.push_back(i);
        uyx.push_back(D.u[N + (size_t)i + (size_t)n * ((size_t)c + (size_t)n * c)] / ulid);
    }
    write_columns(out + "/centerline_ux_y.txt", {y, uxy}, "y  u_x/u_lid at x = z = n/2");
    write_columns(out + "/centerline_uy_x.txt", {x, uyx}, "x  u_y/u_lid at y = z = n/2");
    std::printf("{\"case\": \"cavity\", \"n\": %d, \"steps\": %d, \"seconds\": %.6f, \"mlups\": %.3f, \"last_err\": %.6e}\n",
                n, C.iterations, sec, (double)N * C.iterations / sec / 1e6, C.err);
    return 0;
}

int run_channel(const Args& a) {
    const int nx = a.inum("nx", 256), ny = a.inum("ny", 130), nz = a.inum("nz", 128);
    const double re_tau = a.num("re-tau", 180.0), umax = a.num("umax", 0.05), amp = a.num("amp", 0.05);
    const double h = (ny - 2) / 2.0;
    const double u_tau = umax / 18.3;
    LBMConstants C;
    LBMData D;
    C.dimX_int = nx; C.dimY_int = ny; C.dimZ_int = nz;
    C.ny = u_tau * h / re_tau;
    C.Fx = u_tau * u_tau / h;
    C.CLES = 0.17;
    C.periodic[0] = 1; C.periodic[2] = 1;
    C.iterations = a.inum("steps", 20000);
    C.iterationsMomentAvg = a.inum("avg", C.iterations / 4);
    C.storage = storage_of(a.get("storage", "f32"));
    C.mlp_interval = a.inum("mlp-interval", 1);
    C.plot_every_it = a.inum("plot", -1);
    if (C.plot_every_it > 0) C.results_dir = a.get("out", ".");
    const size_t N = (size_t)nx * ny * nz;
    D.meshFluid.assign(N, 1);
    for (int k = 0; k < nz; k++)
        for (int i = 0; i < nx; i++) {
            D.meshFluid[(size_t)i + (size_t)nx * ((size_t)ny * k)] = 0;
            D.meshFluid[(size_t)i + (size_t)nx * ((size_t)(ny - 1) + (size_t)ny * k)] = 0;
        }
    check(lbm_mesher_wall_pass(D.meshFluid.data(), nx, ny, nz), nullptr, "lbm_mesher_wall_pass");
    D.rhoInit.assign(N, 1.0);
    D.uInit.assign(3 * N, 0.0);
    const uint64_t seed = 0x5EED2026ull;
    const double yc = (ny - 1) / 2.0;
    for (size_t q = 0; q < N; q++) {
        const int j = (int)((q / nx) % ny);
        if (D.meshFluid[q] == 0) continue;
        const double prof = umax * (1.0 - ((j - yc) / h) * ((j - yc) / h));
        for (int c = 0; c < 3; c++) D.uInit[c * N + q] = (uniform01(seed, q, c) * 2.0 - 1.0) * amp * umax;
        D.uInit[q] += prof;
    }
    lbm_mlp_model model{};
    const std::string mlp = a.get("mlp", "");
    if (!mlp.empty()) {
        FILE* f = std::fopen(mlp.c_str(), "rb");
        if (!f || std::fread(&model, sizeof(model), 1, f) != 1) throw Error(LBM_ERR_IO, "cannot read " + mlp);
        std::fclose(f);
        C.mlp = &model;
    }
    double sec = 0.0;
    if (mlp.empty()) {
        SolverTurbulentLES<D3Q27, InitializationEquilibriumConstVector, CollisionCumD3Q27Turbulent2015, StreamingAB,
                           BounceBackWallHalf, NoSymmetry, Periodic, InletVelocityMovingWall, OutletDensityInterpolated,
                           MomentDensityVelocityN27, OmegaLES, ErrorQuadratic, NonDimensiolnaliseFactorsVelocity,
                           MomentTimeAvg>
            s(C, D);
        s.initializeSimulation(true);
        sec = timed_run(s);
    } else {
        SolverTurbulentLES<D3Q27, InitializationEquilibriumConstVector, CollisionCumD3Q27Turbulent2015, StreamingAB,
                           BounceBackWallHalf, NoSymmetry, Periodic, InletVelocityMovingWall, OutletDensityInterpolated,
                           MomentDensityVelocityN27, OmegaMLP, ErrorQuadratic, NonDimensiolnaliseFactorsVelocity,
                           MomentTimeAvg>
            s(C, D);
        s.initializeSimulation(true);
        sec = timed_run(s);
    }
    // plane averages over x and z of the time averages
    std::vector<double> y(ny), mu(ny, 0.0), rxx(ny, 0.0), ryy(ny, 0.0), rzz(ny, 0.0), rxy(ny, 0.0);
    const bool have = !D.uTimeAvg.empty();
    for (int j = 0; j < ny; j++) {
        y[j] = j;
        if (!have) continue;
        double s_u = 0, s_xx = 0, s_yy = 0, s_zz = 0, s_xy = 0;
        for (int k = 0; k < nz; k++)
            for (int i = 0; i < nx; i++) {
                const size_t q = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
                const double ux = D.uTimeAvg[q], uy = D.uTimeAvg[N + q], uz = D.uTimeAvg[2 * N + q];
                s_u += ux;
                s_xx += D.uuTimeAvg[q] - ux * ux;
                s_yy += D.uuTimeAvg[N + q] - uy * uy;
                s_zz += D.uuTimeAvg[2 * N + q] - uz * uz;
                s_xy += D.uuTimeAvg[3 * N + q] - ux * uy;
            }
        const double m = 1.0 / ((double)nx * nz);
        mu[j] = s_u * m; rxx[j] = s_xx * m; ryy[j] = s_yy * m; rzz[j] = s_zz * m; rxy[j] = s_xy * m;
    }
    const std::string out = a.get("out", ".");
    write_columns(out + "/mean_profile.txt", {y, mu, rxx, ryy, rzz, rxy},
                  "y  <u_x>  <u_x'u_x'>  <u_y'u_y'>  <u_z'u_z'>  <u_x'u_y'>  (x, z and time averages)");
    std::printf("{\"case\": \"channel\", \"nx\": %d, \"ny\": %d, \"nz\": %d, \"steps\": %d, \"seconds\": %.6f, "
                "\"glups\": %.4f}\n",
                nx, ny, nz, C.iterations, sec, (double)N * C.iterations / sec / 1e9);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2 || !std::strcmp(argv[1], "--help") || !std::strcmp(argv[1], "-h")) {
        std::printf("usage: lbm_run cavity|channel [--key value ...]  (see the header of lbm_run.cpp)\n"
                    "library ABI version %d\n", lbm_abi_version());
        return argc < 2 ? 2 : 0;
    }
    Args a;
    for (int i = 2; i + 1 < argc; i += 2) {
        if (std::strncmp(argv[i], "--", 2) != 0) {
            std::fprintf(stderr, "unexpected argument %s\n", argv[i]);
            return 2;
        }
        a.kv[argv[i] + 2] = argv[i + 1];
    }
    try {
        if (!std::strcmp(argv[1], "cavity")) return run_cavity(a);
        if (!std::strcmp(argv[1], "channel")) return run_channel(a);
        std::fprintf(stderr, "unknown case %s\n", argv[1]);
        return 2;
    } catch (const Error& e) {
        std::fprintf(stderr, "lbm_run: %s (status %d)\n", e.what(), (int)e.status);
        return 1;
    }
}
