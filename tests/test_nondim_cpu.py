"""NonDimensiolnaliseFactorsVelocity (nonDimensionalisions/NonDimensiolnaliseFactorsVelocity.h:20-130) and
initializeSimulationData (SolverTurbulentLES.h:276-323) of the host mirrors, on the CPU: the factors
restated here in double agree with the mirrors' float arithmetic to float precision, the C++ and the
Python mirrors agree bit for bit, and the checks the reference asserts raise."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from lb_gb300 import capi
from lb_gb300.solver import (NonDimensiolnaliseFactorsVelocity as ND, SolverTurbulentLES)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# physical inputs of the shape main.cu:142-152 sets (air, U_lb = 0.09), on a 1 m x 0.5 m x 0.5 m box
PHYS = dict(BBmin=(0.0, 0.0, 0.0), BBmax=(1.0, 0.5, 0.5), conversion_factor_fyz=1.0, u_guess_fyz=4.0, U_lb=0.09,
            rho_fyz=1.293, ny_fyz=2e-4)
NX = 128


def test_factors_follow_the_definitions():
    c = ND.nonDimensionalize(dict(PHYS), NX)
    Cl = 1.0 / NX
    Cu = 4.0 / 0.09
    Ct = Cl / Cu
    nu = 2e-4 * Ct / Cl ** 2
    ref = dict(L_fyz=1.0, Cl=Cl, Cu=Cu, Cu_inverse=1 / Cu, Ct=Ct, Crho=1.293, Cm=1.293 * Cl ** 3,
               Cpressure=1.293 * Cl ** 3 / Cl / Ct ** 2, Re=4.0 * 1.0 / 2e-4, nu=nu, tau=3 * nu + 0.5,
               omega=1 / (3 * nu + 0.5))
    for k, v in ref.items():
        assert abs(c[k] - v) <= 3e-7 * abs(v), (k, c[k], v)
    r = ND.nonDimensionalize(dict(PHYS, tau_ref_compat=True), NX)
    assert abs(r["tau"] - (nu / 3 + 0.5)) <= 3e-7 and r["tau"] < c["tau"]


def test_reference_asserts_raise():
    with pytest.raises(ValueError):
        ND.nonDimensionalize(dict(PHYS, U_lb=0.6), NX)  # above cs = 0.577
    with pytest.raises(ValueError):
        ND.nonDimensionalize(dict(PHYS, ny_fyz=0.5), NX)  # tau = 4.8


def test_records_and_initial_state_convert():
    c = ND.nonDimensionalize(dict(PHYS), NX)
    ins = ND.nonDimensionalizeInlet([capi.make_inlet(0, 1, 2, (-1, 0, 0), (1.5, 0.0, -0.25))], c)
    assert ins[0].velocity[0] == pytest.approx(1.5 / c["Cu"], rel=1e-6)
    assert ins[0].velocity[2] == pytest.approx(-0.25 / c["Cu"], rel=1e-6)
    assert (ins[0].vertex.x, ins[0].vertex.y, ins[0].vertex.z, ins[0].normal[0]) == (0, 1, 2, -1.0)
    outs = ND.nonDimensionalizeOutlet([capi.make_outlet(9, 1, 2, (1, 0, 0), 1.293)], c)
    assert outs[0].density == pytest.approx(1.0, rel=1e-6)


def test_simulation_data_step_counts_and_probe():
    flags = np.ones((8, 16, NX), np.int32)
    c = dict(PHYS, nu=0.0, plot_every=0.05, err_every_it=100, time=0.5, probe_every_it=10,
             ProbeLocation=(0.5, 0.25, 0.125), additional_factor=0.0, resolution_factor=1.0)
    s = SolverTurbulentLES(constants=c, data={"flags": flags})
    s.convertToLattice()
    s.initializeSimulationData()
    f = np.float32
    assert c["plot_every_it"] == int(np.ceil(f(0.05) / f(c["Ct"])))
    assert c["err_every_it"] == 100
    assert c["iterations"] == int(np.ceil(f(0.5) / f(c["Ct"])))
    # x: 0.5 / 1.0 * 128 = 64; y: 0.25 / 0.5 * 16 = 8; z: 0.125 / 0.5 * 8 = 2
    assert c["ProbeLocationLat"] == (64, 8, 2)
    with pytest.raises(ValueError):
        SolverTurbulentLES(constants=dict(c, plot_every_it=-1, plot_every=-1), data={"flags": flags}) \
            .initializeSimulationData()
    bad = dict(c, ProbeLocation=(1.5, 0.25, 0.125))
    with pytest.raises(ValueError):
        SolverTurbulentLES(constants=bad, data={"flags": flags}).initializeSimulationData()


def test_cpp_mirror_matches_python_bit_for_bit(built_lib):
    src = r'''
#include <cstdio>
#include "lbm_solver.hpp"
using namespace lbm_gb300;
int main() {
    LBMConstants C;
    C.dimX_int = %d;
    C.BBmin[0] = 0.0; C.BBmax[0] = 1.0; C.conversion_factor_fyz = 1.0;
    C.u_guess_fyz = 4.0; C.U_lb = 0.09; C.rho_fyz = 1.293; C.ny_fyz = 2e-4;
    NonDimensiolnaliseFactorsVelocity::nonDimensionalize(C);
    std::printf("%%.9g %%.9g %%.9g %%.9g %%.9g %%.9g %%.9g %%.9g %%.9g\n", C.Cl, C.Cu, C.Ct, C.Cm, C.Cpressure, C.Re, C.ny,
                C.tau, C.omega);
    C.tau_ref_compat = true;
    NonDimensiolnaliseFactorsVelocity::nonDimensionalize(C);
    std::printf("%%.9g\n", C.tau);
    LBMConstants K;
    K.dimX_int = %d; K.dimY_int = 16; K.dimZ_int = 8;
    K.BBmin[0] = 0.0; K.BBmax[0] = 1.0; K.BBmax[1] = 0.5; K.BBmax[2] = 0.5; K.conversion_factor_fyz = 1.0;
    K.u_guess_fyz = 4.0; K.U_lb = 0.09; K.rho_fyz = 1.293; K.ny_fyz = 2e-4;
    K.plot_every = 0.05; K.err_every_it = 100; K.time = 0.5; K.probe_every_it = 10;
    K.ProbeLocation[0] = 0.5; K.ProbeLocation[1] = 0.25; K.ProbeLocation[2] = 0.125;
    K.additional_factor = 0.0; K.resolution_factor = 1.0;
    LBMData D;
    SolverTurbulentLES<D3Q27, InitializationEquilibriumConstVector, CollisionCumD3Q27Turbulent2015, StreamingAB,
                       BounceBackWallHalf, NoSymmetry, Periodic, InletVelocityEquilibrium,
                       OutletDensityInterpolated, MomentDensityVelocityN27, OmegaLES, ErrorQuadratic,
                       NonDimensiolnaliseFactorsVelocity, MomentTimeAvg> s(K, D);
    s.convertToLattice(false);
    s.initializeSimulationData(false);
    std::printf("%%d %%d %%d %%d %%d %%d\n", K.plot_every_it, K.err_every_it, K.iterations, K.ProbeLocationLat[0],
                K.ProbeLocationLat[1], K.ProbeLocationLat[2]);
    return 0;
}
''' % (NX, NX)
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "t.cpp")
        exe = os.path.join(d, "t")
        with open(p, "w") as fh:
            fh.write(src)
        lib = os.path.join(ROOT, "lb_gb300")
        r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), p,
                            "-L", lib, "-llbm_gb300", "-Wl,-rpath," + lib, "-o", exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    c = ND.nonDimensionalize(dict(PHYS), NX)
    want = [c[k] for k in ("Cl", "Cu", "Ct", "Cm", "Cpressure", "Re", "nu", "tau", "omega")]
    want.append(ND.nonDimensionalize(dict(PHYS, tau_ref_compat=True), NX)["tau"])
    assert [float(v) for v in out[:10]] == [float("%.9g" % w) for w in want]
    k = dict(PHYS, nu=0.0, plot_every=0.05, err_every_it=100, time=0.5, probe_every_it=10,
             ProbeLocation=(0.5, 0.25, 0.125), additional_factor=0.0, resolution_factor=1.0)
    s = SolverTurbulentLES(constants=k, data={"flags": np.ones((8, 16, NX), np.int32)})
    s.convertToLattice()
    s.initializeSimulationData()
    assert [int(v) for v in out[10:]] == [k["plot_every_it"], k["err_every_it"], k["iterations"],
                                          *k["ProbeLocationLat"]]


def test_laminar_solver_sets_up_like_the_reference():
    """SolverLaminar (SolverLaminar.h:94-125): no turbulence policy (OmegaNo), and initializeSimulation runs
    initializeSimulationData first, so missing output intervals are refused before the GPU is touched."""
    from lb_gb300.solver import OmegaNo, SolverLaminar
    flags = np.ones((4, 5, 6), np.int32)
    s = SolverLaminar(constants=dict(nu=0.1, err_every_it=10), data={"flags": flags})
    assert s.policies["Turbulence"] is OmegaNo
    with pytest.raises(ValueError, match="plot_every"):
        s.initializeSimulation()


@pytest.mark.parametrize("laminar", [False, True])
def test_step_schedule_replays_the_reference_loop(laminar):
    """step_schedule (the Python mirror's runSimulation) against the reference loop run step by step
    (SolverTurbulentLES.h:184-253, SolverLaminar.h:131-175): the same events after the same steps and the
    same averaged states."""
    from lb_gb300.solver import step_schedule
    rng = np.random.default_rng(5)
    for _ in range(300):
        it = int(rng.integers(1, 60))
        avg = int(rng.integers(0, it + 1))
        kw = dict(err_every=int(rng.choice([-1, 1, 3, 10])), probe_every=int(rng.choice([-1, 1, 4])),
                  probe_iterations=int(rng.integers(0, 70)), plot_every=int(rng.choice([-1, 1, 5, 7])))
        naive_events, naive_avg = [], set()
        for k in range(it):
            if k > it - avg:
                naive_avg.add(k)
            ev = []
            if not laminar and kw["probe_every"] > 0 and k % kw["probe_every"] == 0 and k >= it - kw["probe_iterations"]:
                ev.append("probe")
            if kw["err_every"] > 0 and k % kw["err_every"] == 0 and k != 0:
                ev.append("err")
            if kw["plot_every"] > 0 and k % kw["plot_every"] == 0 and (k != 0 or laminar):
                ev.append("plot")
            if ev:
                naive_events.append((k, tuple(ev)))
        sched = step_schedule(it, avg, laminar=laminar, **kw)
        assert sum(n for _, n, _, _ in sched) == it
        assert [(j, ev) for _, _, j, ev in sched if ev] == naive_events
        averaged, on, done = set(), False, 0
        for begin, n, j, _ in sched:
            on = on or begin
            if on:
                averaged.update(range(done, done + n))
            done += n
        assert averaged == naive_avg, (it, avg)


class _FakeSolver:
    """Stands in for the GPU Solver under SolverTurbulentLES.runSimulation: counts steps, records when
    each call happens and returns fields that depend on the step count."""

    def __init__(self, shape):
        self.shape = shape
        self.N = shape[0] * shape[1] * shape[2]
        self.k = 0
        self.calls = []

    def step(self, n):
        self.k += n

    def timeavg_begin(self):
        self.calls.append(("avg_begin", self.k))

    def timeavg_end(self):
        self.calls.append(("avg_end", self.k))

    def timeavg_get(self):
        return np.full(self.N, 1.0), np.zeros((3, self.N)), None, None

    def probe(self, x, y, z):
        self.calls.append(("probe", self.k, (x, y, z)))
        return np.array([0.01, 0.0, 0.0, 1.0])

    def error_evaluation(self):
        self.calls.append(("err", self.k))
        return 1.0 / self.k

    def moments(self):
        return np.full(self.N, 1.0 + 1e-3 * self.k), np.zeros((3, self.N))


@pytest.mark.parametrize("laminar", [False, True])
def test_python_run_loop_calls_and_files(tmp_path, laminar):
    """SolverTurbulentLES.runSimulation (and SolverLaminar's) on a stand-in solver: the average starts
    after it - avg + 1 steps, errors come after steps k = 10, 20 (k + 1 steps done), dumps and probe lines
    land under results_dir with the reference's names."""
    from lb_gb300.solver import SolverLaminar
    shape = (4, 3, 2)
    c = dict(nu=0.1, iterations=25, iterationsMomentAvg=5, err_every_it=10, plot_every_it=7, probe_every_it=4,
             probe_iterations=9, ProbeLocationLat=(1, 1, 0), results_dir=str(tmp_path))
    cls = SolverLaminar if laminar else SolverTurbulentLES
    s = cls(constants=c, data={"flags": np.ones(shape[::-1], np.int32)})
    s.solver = _FakeSolver(shape)
    errors = s.runSimulation()
    assert s.solver.k == 25
    assert [e[0] for e in errors] == [10, 20]
    calls = s.solver.calls
    assert ("avg_begin", 21) in calls and calls[-1] == ("avg_end", 25)
    assert [cl[1] for cl in calls if cl[0] == "err"] == [11, 21]
    probes = [cl[1] for cl in calls if cl[0] == "probe"]
    assert probes == ([] if laminar else [17, 21, 25])  # after steps k = 16, 20, 24 (k >= 25 - 9)
    files = sorted(p.name for p in tmp_path.iterdir())
    if laminar:
        assert files == ["variablesLattice0.vtk", "variablesLattice1.vtk", "variablesLattice2.vtk",
                         "variablesLattice3.vtk", "variablesTimeAvg.vtk"]
    else:
        assert files == ["probeData.csv", "variables.1.vtk", "variables.2.vtk", "variables.3.vtk",
                         "variablesTimeAvg.vtk"]
        assert len((tmp_path / "probeData.csv").read_text().splitlines()) == 2 + 3
