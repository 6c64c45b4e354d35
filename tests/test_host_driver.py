"""The C++ host side: include/lbm_solver.hpp (the reference's SolverTurbulentLES policy interface over the
C ABI) and the driver lb_gb300/host/lbm_run.cpp built on it."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from lb_gb300 import build, cases
from lb_gb300.solver import OmegaLES, OmegaNo, Solver

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_driver_is_built_and_reports_the_abi(built_lib):
    r = subprocess.run([build.DRIVER, "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0
    assert "ABI version 3" in r.stdout


def test_unsupported_policy_does_not_compile():
    """A policy the fused kernel does not implement is a compile error, not a silent substitute."""
    src = r'''
#include "lbm_solver.hpp"
using namespace lbm_gb300;
struct BounceSymmetryFull {};
int main() {
    LBMConstants C; LBMData D;
    SolverTurbulentLES<D3Q27, InitializationEquilibriumConstVector, CollisionCumD3Q27Turbulent2015, StreamingAB,
                       BounceBackWallHalf, BounceSymmetryFull, NoPeriodic, InletVelocityMovingWall,
                       OutletDensityInterpolated, MomentDensityVelocityN27, OmegaLES, ErrorQuadratic,
                       NonDimensiolnaliseFactorsVelocity, MomentTimeAvg> s(C, D);
    return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "t.cpp")
        with open(p, "w") as fh:
            fh.write(src)
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), p],
                           capture_output=True, text=True)
    assert r.returncode != 0
    assert "symmetry: NoSymmetry or BounceSymmetryHalf" in r.stderr


def test_supported_policies_compile():
    """Every policy tag the kernels implement composes into SolverTurbulentLES (the reference's
    declaration in main.cu reads the same with these names)."""
    src = r'''
#include "lbm_solver.hpp"
using namespace lbm_gb300;
int main() {
    LBMConstants C; LBMData D;
    SolverTurbulentLES<D3Q27, InitializationEquilibriumConstVector, CollisionCumD3Q27Turbulent2017, StreamingAB,
                       BounceBackWallHalfMesh, BounceSymmetryHalf, Periodic, InletVelocityZouHe,
                       OutletNeighbourEquilibriumOmega, MomentDensityVelocityN27, OmegaLES, ErrorQuadratic,
                       NonDimensiolnaliseFactorsVelocity, MomentTimeAvg> a(C, D);
    SolverTurbulentLES<D3Q27, InitializationEquilibriumConstVector, CollisionCumD3Q27TurbulentCombined, StreamingAB,
                       BounceBackWallHalf, NoSymmetry, NoPeriodic, InletVelocityEquilibrium,
                       OutletDensityEquilibrium, MomentDensityVelocityN27, OmegaNo, ErrorQuadratic,
                       NonDimensiolnaliseFactorsVelocity, MomentTimeAvg> b(C, D);
    SolverTurbulentLES<D3Q27, InitializationEquilibriumConstVector, CollisionSRTTurbulent, StreamingAB,
                       BounceBackWallHalf, NoSymmetry, Periodic, InletVelocityMovingWall,
                       OutletNeighbourEquilibriumOmegaRF, MomentDensityVelocityN27, OmegaMLP, ErrorQuadratic,
                       NonDimensiolnaliseFactorsVelocity, MomentTimeAvg> c(C, D);
    SolverTurbulentLES<D3Q27, InitializationEquilibriumConstVector, CollisionSRTunroll, StreamingAB,
                       BounceBackWallHalf, NoSymmetry, Periodic, InletVelocityZouHe,
                       OutletNeighbourEquilibriumOmega, MomentDensityVelocityN27, OmegaLES, ErrorQuadratic,
                       NonDimensiolnaliseFactorsVelocity, MomentTimeAvg> e(C, D);
    SolverTurbulentLES<D3Q27, InitializationEquilibriumConstVector, CollisionCumD3Q27Laminar, StreamingAB,
                       BounceBackWallHalf, NoSymmetry, NoPeriodic, InletVelocityMovingWall,
                       OutletDensityInterpolated, MomentDensityVelocityN27, OmegaMLP, ErrorQuadratic,
                       NonDimensiolnaliseFactorsVelocity, MomentTimeAvg> f(C, D);
    SolverTurbulentLES<D3Q27, InitializationEquilibriumVariables, CollisionSRTLaminar, StreamingAB,
                       BounceBackWallHalf, NoSymmetry, NoPeriodic, InletVelocityMovingWall,
                       OutletDensityInterpolated, MomentDensityVelocityN27, OmegaNo, ErrorQuadratic,
                       NonDimensiolnaliseFactorsVelocity, MomentTimeAvg> g(C, D);
    SolverLaminar<D3Q27, InitializationEquilibriumConstVector, CollisionCumD3Q27Laminar, StreamingAB,
                  BounceBackWallHalf, NoSymmetry, Periodic, InletVelocityEquilibrium, OutletDensityInterpolated,
                  MomentDensityVelocityN27, ErrorQuadratic, NonDimensiolnaliseFactorsVelocity, MomentTimeAvg> h(C, D);
    static_assert(CollisionSRTunroll::laminar && CollisionCumD3Q27Laminar::laminar &&
                  !CollisionCumD3Q27Turbulent2015::laminar, "laminar tags");
    (void)a; (void)b; (void)c; (void)e; (void)f; (void)g; (void)h;
    return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "t.cpp")
        with open(p, "w") as fh:
            fh.write(src)
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), p],
                           capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_driver_cavity_equals_python_api(built_lib):
    n, steps = 24, 300
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([build.DRIVER, "cavity", "--n", str(n), "--steps", str(steps), "--storage", "f64",
                            "--err-every", "100", "--out", d], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        prof = np.loadtxt(os.path.join(d, "centerline_ux_y.txt"))
    c = cases.cavity(n)
    s = Solver((n, n, n), turbulence=OmegaNo, storage="f64", nu=c["nu"])
    s.set_flags(c["flags"])
    s.set_bc(c["inlets"])
    s.init_equilibrium(1.0, (0.0, 0.0, 0.0))
    s.step(steps)
    _, u = s.moments()
    s.close()
    ux = u[0].reshape(n, n, n)[n // 2, :, n // 2] / 0.05
    assert np.array_equal(prof[:, 1], ux)


@pytest.mark.gpu
def test_driver_writes_the_reference_vtk_dumps(built_lib):
    """runSimulation with plot_every_it = 10 writes variables.1.vtk after step index 10 (11 steps) and
    variables.2.vtk after 21 steps, as SolverTurbulentLES.h:246-252 does; the dumped U equals the Python
    API's state after the same steps to the file's 6 digits."""
    n, steps = 12, 21
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([build.DRIVER, "cavity", "--n", str(n), "--steps", str(steps), "--storage", "f64",
                            "--err-every", "0", "--plot", "10", "--out", d], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        assert sorted(f for f in os.listdir(d) if f.endswith(".vtk")) == ["variables.1.vtk", "variables.2.vtk"]
        lines = open(os.path.join(d, "variables.2.vtk")).read().splitlines()
    N = n ** 3
    assert lines[0] == "# vtk DataFile Version 2.0" and lines[4] == f"DIMENSIONS {n} {n} {n}"
    i = lines.index("VECTORS U double")
    U = np.array([[float(t) for t in l.split()] for l in lines[i + 1:i + 1 + N]]).T
    c = cases.cavity(n)
    s = Solver((n, n, n), turbulence=OmegaNo, storage="f64", nu=c["nu"])
    s.set_flags(c["flags"])
    s.set_bc(c["inlets"])
    s.init_equilibrium(1.0, (0.0, 0.0, 0.0))
    s.step(steps)
    _, u = s.moments()
    s.close()
    assert np.allclose(U, u, rtol=6e-6, atol=1e-12)  # 6 significant digits: up to 5e-6 relative


@pytest.mark.gpu
def test_driver_channel_profile_equals_python_api(built_lib):
    nx, ny, nz, steps, avg = 64, 34, 32, 200, 50
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([build.DRIVER, "channel", "--nx", str(nx), "--ny", str(ny), "--nz", str(nz), "--steps",
                            str(steps), "--avg", str(avg), "--storage", "f32", "--out", d],
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        prof = np.loadtxt(os.path.join(d, "mean_profile.txt"))
    c = cases.channel(nx, ny, nz, re_tau=180.0, u_max=0.05, amp=0.05)
    s = Solver((nx, ny, nz), turbulence=OmegaLES, storage="f32", nu=c["nu"], cles=0.17, periodic=c["periodic"],
               force=c["force"])
    s.set_flags(c["flags"])
    s.set_bc()
    s.init_fields(c["rho"], c["u"])
    s.step(steps - avg + 1)
    s.timeavg_begin()
    s.step(avg - 1)
    s.timeavg_end()
    _, um, uu, _ = s.timeavg_get()
    s.close()
    um = um.reshape(3, nz, ny, nx)
    uu = uu.reshape(6, nz, ny, nx)
    mean_ux = um[0].mean(axis=(0, 2))
    rxy = (uu[3] - um[0] * um[1]).mean(axis=(0, 2))
    assert np.allclose(prof[:, 1], mean_ux, rtol=1e-12, atol=1e-15)
    assert np.allclose(prof[:, 5], rxy, rtol=1e-9, atol=1e-15)


STUB = r'''
// stand-in for the library: records the calls SolverTurbulentLES makes (no GPU)
#include <cstdio>
#include <cstring>
#include "lbm.h"
static int g_k = 0;
static lbm_ctx* const CTX = (lbm_ctx*)0x1;
extern "C" {
lbm_status lbm_create(const lbm_config*, lbm_ctx** c) { *c = CTX; return LBM_OK; }
lbm_status lbm_destroy(lbm_ctx*) { return LBM_OK; }
const char* lbm_last_error(const lbm_ctx*) { return ""; }
const char* lbm_vtk_last_error(void) { return ""; }
lbm_status lbm_set_flags(lbm_ctx*, const int32_t*) { return LBM_OK; }
lbm_status lbm_set_bc(lbm_ctx*, const lbm_bc_inlet*, int32_t, const lbm_bc_outlet*, int32_t) { return LBM_OK; }
lbm_status lbm_set_symmetry(lbm_ctx*, const lbm_bc_symmetry*, int32_t) { return LBM_OK; }
lbm_status lbm_init_equilibrium(lbm_ctx*, double, const double*) { return LBM_OK; }
lbm_status lbm_init_fields(lbm_ctx*, const double*, const double*) { return LBM_OK; }
lbm_status lbm_vtk_read_variables(const char*, const int32_t*, double*, double*) { return LBM_OK; }
lbm_status lbm_mlp_load(lbm_ctx*, const lbm_mlp_model*) { return LBM_OK; }
lbm_status lbm_step(lbm_ctx*, int32_t n) { g_k += n; return LBM_OK; }
lbm_status lbm_synchronize(lbm_ctx*) { return LBM_OK; }
lbm_status lbm_timeavg_begin(lbm_ctx*) { std::printf("avg_begin %d\n", g_k); return LBM_OK; }
lbm_status lbm_timeavg_end(lbm_ctx*) { std::printf("avg_end %d\n", g_k); return LBM_OK; }
lbm_status lbm_timeavg_get(lbm_ctx*, double*, double*, double*, int64_t*) { return LBM_OK; }
lbm_status lbm_probe(lbm_ctx*, int32_t, int32_t, int32_t, double out[4]) {
    std::printf("probe %d\n", g_k); out[0] = out[1] = out[2] = 0; out[3] = 1; return LBM_OK; }
lbm_status lbm_error_evaluation(lbm_ctx*, double* e) { std::printf("err %d\n", g_k); *e = 1.0; return LBM_OK; }
lbm_status lbm_get_moments(lbm_ctx*, double*, double*) { return LBM_OK; }
lbm_status lbm_vtk_write(const char* path, const char*, const int32_t*, double, double, const double*,
                         const lbm_vtk_field*, int32_t) { std::printf("vtk %s %d\n", std::strrchr(path, '/') + 1, g_k);
                                                          return LBM_OK; }
lbm_status lbm_probe_csv_append(const char*, double, const double*, double, double, double) { return LBM_OK; }
}
'''


@pytest.mark.parametrize("laminar", [False, True])
def test_cpp_run_loop_matches_the_python_schedule(laminar):
    """SolverTurbulentLES / SolverLaminar::runSimulation of include/lbm_solver.hpp, linked against a
    stand-in library that records the calls: the average, probe, error and dump calls come after the same
    steps as in step_schedule (the Python mirror's loop, itself checked against the reference loop)."""
    from lb_gb300.solver import step_schedule
    it, avg, err, plot, probe, probe_its = 25, 5, 10, 7, 4, 9
    solver = ("SolverLaminar<D3Q27, InitializationEquilibriumConstVector, CollisionCumD3Q27Laminar, StreamingAB, "
              "BounceBackWallHalf, NoSymmetry, NoPeriodic, InletVelocityMovingWall, OutletDensityInterpolated, "
              "MomentDensityVelocityN27, ErrorQuadratic, NonDimensiolnaliseFactorsVelocity, MomentTimeAvg>"
              if laminar else
              "SolverTurbulentLES<D3Q27, InitializationEquilibriumConstVector, CollisionCumD3Q27Turbulent2015, "
              "StreamingAB, BounceBackWallHalf, NoSymmetry, NoPeriodic, InletVelocityMovingWall, "
              "OutletDensityInterpolated, MomentDensityVelocityN27, OmegaLES, ErrorQuadratic, "
              "NonDimensiolnaliseFactorsVelocity, MomentTimeAvg>")
    main = r'''
#include "lbm_solver.hpp"
using namespace lbm_gb300;
int main() {
    LBMConstants C; LBMData D;
    C.dimX_int = 4; C.dimY_int = 3; C.dimZ_int = 2; D.meshFluid.assign(24, 1);
    C.iterations = %d; C.iterationsMomentAvg = %d; C.err_every_it = %d; C.plot_every_it = %d;
    C.probe_every_it = %d; C.probe_iterations = %d; C.results_dir = "out";
    %s s(C, D);
    s.initializeSimulation(false);
    s.runSimulation();
    return 0;
}
''' % (it, avg, err, plot, probe, probe_its, solver)
    with tempfile.TemporaryDirectory() as d:
        for name, text in (("stub.cpp", STUB), ("main.cpp", main)):
            with open(os.path.join(d, name), "w") as fh:
                fh.write(text)
        exe = os.path.join(d, "t")
        r = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), os.path.join(d, "main.cpp"),
                            os.path.join(d, "stub.cpp"), "-o", exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines()
    want = []
    for begin, n, j, events in step_schedule(it, avg, err_every=err, probe_every=probe, probe_iterations=probe_its,
                                             plot_every=plot, laminar=laminar):
        done = j + 1
        if begin:
            want.append(f"avg_begin {done - n}")
        for e in events:
            if e == "probe":
                want.append(f"probe {done}")
            elif e == "err":
                want.append(f"err {done}")
            else:
                name = f"variablesLattice{j // plot}.vtk" if laminar else f"variables.{j // plot}.vtk"
                want.append(f"vtk {name} {done}")
    want += [f"avg_end {it}", f"vtk variablesTimeAvg.vtk {it}"]
    assert out == want


SETUP_STUB = STUB.replace(
    "lbm_status lbm_create(const lbm_config*, lbm_ctx** c) { *c = CTX; return LBM_OK; }",
    "lbm_status lbm_create(const lbm_config* g, lbm_ctx** c) { *c = CTX; std::printf(\"cfg %d %d %d %d %.9g %.9g "
    "%g %g %d%d%d\\n\", g->collision, g->closure, g->inlet_kind, g->outlet_kind, g->nu, g->tau, g->omega_dumping_low, "
    "g->omega_dumping_high, g->periodic[0], g->periodic[1], g->periodic[2]); return LBM_OK; }").replace(
    "lbm_status lbm_set_bc(lbm_ctx*, const lbm_bc_inlet*, int32_t, const lbm_bc_outlet*, int32_t) { return LBM_OK; }",
    "lbm_status lbm_set_bc(lbm_ctx*, const lbm_bc_inlet* i, int32_t ni, const lbm_bc_outlet* o, int32_t no) { "
    "for (int e = 0; e < ni; e++) std::printf(\"inlet %.9g\\n\", i[e].velocity[0]); "
    "for (int e = 0; e < no; e++) std::printf(\"outlet %.9g\\n\", o[e].density); return LBM_OK; }").replace(
    "lbm_status lbm_init_equilibrium(lbm_ctx*, double, const double*) { return LBM_OK; }",
    "lbm_status lbm_init_equilibrium(lbm_ctx*, double r, const double* u) { std::printf(\"init %.9g %.9g\\n\", r, u[0]); "
    "return LBM_OK; }").replace(
    "lbm_status lbm_vtk_read_variables(const char*, const int32_t*, double*, double*) { return LBM_OK; }",
    "lbm_status lbm_vtk_read_variables(const char* p, const int32_t*, double*, double*) { std::printf(\"read %s\\n\", p); "
    "return LBM_OK; }").replace(
    "lbm_status lbm_init_fields(lbm_ctx*, const double*, const double*) { return LBM_OK; }",
    "lbm_status lbm_init_fields(lbm_ctx*, const double*, const double*) { std::printf(\"init_fields\\n\"); "
    "return LBM_OK; }")


def run_setup(solver, body):
    main = r'''
#include "lbm_solver.hpp"
using namespace lbm_gb300;
int main() {
    LBMConstants C; LBMData D;
    C.dimX_int = 4; C.dimY_int = 3; C.dimZ_int = 2; D.meshFluid.assign(24, 1);
    C.periodic[0] = 1; C.omegaDumpingLow = 0.0; C.omegaDumpingHigh = 0.05;
    lbm_bc_inlet in{}; in.velocity[0] = 4.0f; D.meshBoundaryInlet.push_back(in);
    lbm_bc_outlet out{}; out.density = 1.293f; D.meshBoundaryOutlet.push_back(out);
    %s
    %s s(C, D);
    s.convertToLattice(false);
    s.initializeSimulation(false);
    return 0;
}
''' % (body, solver)
    with tempfile.TemporaryDirectory() as d:
        for name, text in (("stub.cpp", SETUP_STUB), ("main.cpp", main)):
            with open(os.path.join(d, name), "w") as fh:
                fh.write(text)
        exe = os.path.join(d, "t")
        r = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), os.path.join(d, "main.cpp"),
                            os.path.join(d, "stub.cpp"), "-o", exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        return subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines()


TAGS = ("D3Q27, {init}, {coll}, StreamingAB, BounceBackWallHalf, NoSymmetry, Periodic, InletVelocityEquilibrium, "
        "OutletNeighbourEquilibriumOmega, MomentDensityVelocityN27, {turb}ErrorQuadratic, "
        "NonDimensiolnaliseFactorsVelocity, MomentTimeAvg")


def test_cpp_setup_converts_physical_inputs():
    """convertToLattice + initializeSimulation of the C++ mirror (stand-in library): the config carries the
    converted nu and tau, the inlet velocity is divided by Cu, the outlet density by Crho, and the initial
    state is rho_fyz / Crho with VelocityInit / Cu (InitializationEquilibriumConstVector.h:79-82)."""
    from lb_gb300.solver import NonDimensiolnaliseFactorsVelocity as ND
    phys = ("C.ny_fyz = 2e-4; C.rho_fyz = 1.293; C.u_guess_fyz = 4.0; C.U_lb = 0.09; C.BBmax[0] = 1.0; "
            "C.VelocityInit[0] = 2.0;")
    out = run_setup("SolverTurbulentLES<%s>" % TAGS.format(init="InitializationEquilibriumConstVector",
                                                          coll="CollisionCumD3Q27Turbulent2015", turb="OmegaLES, "),
                    phys)
    c = ND.nonDimensionalize(dict(BBmin=(0, 0, 0), BBmax=(1.0, 0, 0), u_guess_fyz=4.0, U_lb=0.09, rho_fyz=1.293,
                                  ny_fyz=2e-4), 4)
    cfg = out[0].split()
    assert cfg[1:5] == ["1", "1", "1", "2"] and cfg[-1] == "100"
    assert float(cfg[5]) == pytest.approx(c["nu"], rel=1e-7) and float(cfg[6]) == pytest.approx(c["tau"], rel=1e-7)
    assert (cfg[7], cfg[8]) == ("0", "0.05")
    assert float(out[1].split()[1]) == pytest.approx(4.0 / c["Cu"], rel=1e-6)
    assert float(out[2].split()[1]) == pytest.approx(1.0, rel=1e-6)
    init = out[3].split()
    assert float(init[1]) == pytest.approx(1.0, rel=1e-6) and float(init[2]) == pytest.approx(2.0 / c["Cu"], rel=1e-6)


def test_cpp_setup_laminar_and_restart_choices():
    """A laminar collision runs without closure and sponge; SolverLaminar drops the periodic axes (its loop
    has no periodic hook); InitializationEquilibriumVariables reads results/<InitFileName>."""
    out = run_setup("SolverTurbulentLES<%s>" % TAGS.format(init="InitializationEquilibriumVariables",
                                                          coll="CollisionSRTLaminar", turb="OmegaLES, "),
                    'C.InitFileName = "variablesLattice3.vtk";')
    cfg = out[0].split()
    assert cfg[1:3] == ["0", "0"] and (cfg[7], cfg[8]) == ("0", "0") and cfg[-1] == "100"
    assert out[1:] == ["inlet 4", "outlet 1.29299998", "read results/variablesLattice3.vtk", "init_fields"]
    lam = TAGS.format(init="InitializationEquilibriumConstVector", coll="CollisionCumD3Q27Turbulent2015", turb="")
    out = run_setup("SolverLaminar<%s>" % lam, "C.plot_every_it = 10; C.err_every_it = 10;")
    cfg = out[0].split()
    assert cfg[1:3] == ["1", "0"] and cfg[-1] == "000"
