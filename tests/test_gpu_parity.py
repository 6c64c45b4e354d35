"""GPU kernels (through the C ABI) against the CPU oracle on the same seeded inputs.

Tolerances (stated per test): FP64 GPU vs FP64 oracle <= 1e-12 relative; FP32 GPU vs FP32 oracle
per-cell |du| <= 1e-5 of the velocity scale after 100 steps; FP16-deviation storage against the
FP64 oracle with a bound set by the 2^-10 storage quantum.  Moments are compared, never raw
populations (the AA layout stores shifted slots on odd steps).
"""
import os

import numpy as np
import pytest

from lb_gb300 import capi, cases
from lb_gb300.solver import (CollisionCumD3Q27Turbulent2015, CollisionCumD3Q27Turbulent2017,
                             CollisionCumD3Q27TurbulentCombined, CollisionSRTTurbulent, InletVelocityEquilibrium,
                             InletVelocityMovingWall, OmegaLES, OmegaNo, Solver)
from oracle import oracle as O

pytestmark = pytest.mark.gpu

COLL = {"cum": CollisionCumD3Q27Turbulent2015, "cum17": CollisionCumD3Q27Turbulent2017,
        "comb": CollisionCumD3Q27TurbulentCombined, "srt": CollisionSRTTurbulent}
CLOS = {"smag": OmegaLES, "none": OmegaNo}


def pair(shape, case, coll, clos, storage, prec, inlet=InletVelocityMovingWall, periodic=None, force=(0, 0, 0)):
    periodic = case.get("periodic", (0, 0, 0)) if periodic is None else periodic
    g = Solver(shape, collision=COLL[coll], turbulence=CLOS[clos], inlet=inlet, storage=storage, nu=case["nu"],
               cles=0.17, periodic=periodic, force=force)
    g.set_flags(case["flags"])
    g.set_bc(case["inlets"], case["outlets"])
    cfg = capi.make_config(*shape, periodic=periodic, collision=COLL[coll].code, closure=CLOS[clos].code,
                           inlet_kind=inlet.code, nu=case["nu"], cles=0.17, force=force)
    o = O.OracleSim(cfg, prec)
    o.set_flags(case["flags"])
    o.set_bc(case["inlets"], case["outlets"])
    return g, o


def init_both(g, o, case, rho0=1.0, u0=(0, 0, 0)):
    if "rho" in case:
        g.init_fields(case["rho"], case["u"])
        o.init_fields(case["rho"], case["u"])
    else:
        g.init_equilibrium(rho0, u0)
        o.init_equilibrium(rho0, u0)


def compare(g, o, uscale, tol_rho, tol_u, mask=None):
    rg, ug = g.moments()
    ro, uo = o.moments()
    if mask is not None:
        rg, ro, ug, uo = rg[mask], ro[mask], ug[:, mask], uo[:, mask]
    dr = np.abs(rg - ro).max()
    du = np.abs(ug - uo).max() / uscale
    assert dr <= tol_rho, (dr, tol_rho)
    assert du <= tol_u, (du, tol_u)
    return dr, du


@pytest.mark.parametrize("coll,clos", [("cum", "smag"), ("cum", "none"), ("cum17", "smag"), ("cum17", "none"),
                                       ("comb", "smag"), ("srt", "smag"), ("srt", "none")])
def test_cavity_fp64_matches_oracle(built_lib, oracle_lib, coll, clos):
    n = 20
    c = cases.cavity(n, u_lid=0.05, re=400.0)
    g, o = pair((n, n, n), c, coll, clos, "f64", 64)
    init_both(g, o, c)
    for _ in range(4):
        g.step(25)
        o.step(25)
        compare(g, o, 0.05, 1e-12, 1e-12)


@pytest.mark.parametrize("coll,re", [("cum", 1000.0), ("cum17", 1000.0), ("comb", 1000.0), ("srt", 400.0),
                                     ("srt", 1000.0)])
def test_cavity_fp32_matches_oracle_fp32(built_lib, oracle_lib, coll, re):
    """FP32 parity after 100 steps at tau = 0.5036 / 0.509.  The FP32 oracle itself drifts
    0.9-1.4e-5 (of u_lid) from the FP64 oracle here (rounding noise that over-relaxation at
    tau -> 1/2 amplifies), so the bar is: GPU FP32 within 3e-5 of the FP32 oracle, and no farther
    from the FP64 oracle than 1.5x the FP32 oracle's own distance (+1e-6)."""
    n = 24
    c = cases.cavity(n, u_lid=0.05, re=re)
    g, o = pair((n, n, n), c, coll, "smag", "f32", 32)
    _, o64 = pair((n, n, n), c, coll, "smag", "f64", 64)
    init_both(g, o, c)
    o64.init_equilibrium(1.0, (0, 0, 0))
    fp32_parity(g, o, o64, 0.05, 100)


def fp32_parity(g, o, o64, uscale, steps):
    """FP32 GPU vs FP32 oracle: within 3e-5 of the velocity scale, and no farther from the FP64
    oracle than 1.5x the FP32 oracle's own distance (+1e-6): the FP32 rounding-noise floor of these
    cases after 100 steps is 0.9e-5 to 2.4e-5, measured as |FP32 oracle - FP64 oracle|."""
    g.step(steps)
    o.step(steps)
    o64.step(steps)
    compare(g, o, uscale, 3e-5, 3e-5)
    _, ug = g.moments()
    _, uo = o.moments()
    _, ut = o64.moments()
    e_gpu = np.abs(ug - ut).max() / uscale
    e_orc = np.abs(uo - ut).max() / uscale
    assert e_gpu <= 1.5 * e_orc + 1e-6, (e_gpu, e_orc)


@pytest.mark.parametrize("coll", ["cum", "cum17", "comb"])
def test_channel_periodic_force_fp64(built_lib, oracle_lib, coll):
    nx, ny, nz = 24, 14, 12
    c = cases.channel(nx, ny, nz, re_tau=3.0, u_max=0.05, nu=0.01)  # u_tau = 0.005, F = 4e-6
    g, o = pair((nx, ny, nz), c, coll, "smag", "f64", 64, force=c["force"])
    init_both(g, o, c)
    for _ in range(3):
        g.step(33)
        o.step(33)
        compare(g, o, 0.05, 1e-12, 1e-12)


@pytest.mark.parametrize("storage", ["f32", "f16dev"])
@pytest.mark.parametrize("coll", ["cum", "cum17", "comb"])
def test_channel_packed_pairs(built_lib, oracle_lib, storage, coll):
    """Periodic channel with force on an even-width lattice: interior cells run the packed
    two-cell path, the seams and wall rows the per-cell path."""
    nx, ny, nz = 32, 14, 12
    c = cases.channel(nx, ny, nz, re_tau=3.0, u_max=0.05, nu=0.01)
    g, o = pair((nx, ny, nz), c, coll, "smag", storage, 32, force=c["force"])
    _, o64 = pair((nx, ny, nz), c, coll, "smag", "f64", 64, force=c["force"])
    init_both(g, o, c)
    o64.init_fields(c["rho"], c["u"])
    if storage == "f32":
        fp32_parity(g, o, o64, 0.05, 100)
    else:  # FP16-deviation storage: relative L2 of u against FP64
        g.step(100)
        o64.step(100)
        _, ug = g.moments()
        _, ut = o64.moments()
        fl = c["flags"].reshape(-1) != 0
        assert np.linalg.norm(ug[:, fl] - ut[:, fl]) / np.linalg.norm(ut[:, fl]) < 2e-3


@pytest.mark.parametrize("shape,case_kind", [((64, 14, 12), "channel"), ((64, 8, 6), "box"), ((128, 6, 5), "box")])
def test_row_staged_step_is_bit_identical_to_per_pair_path(built_lib, shape, case_kind):
    """FP16-deviation storage, periodic x: rows of bulk cells go through the shared-memory
    row-staged kernel (cp.async.bulk in and out) when LBM_OPT_ROW_STAGING is set, the rest through
    the per-pair path.  The default per-pair path everywhere must give the same populations bit for bit,
    on odd and even steps, including rows on the periodic y/z seams of a fully periodic box."""
    nx, ny, nz = shape
    if case_kind == "channel":
        c = cases.channel(nx, ny, nz, re_tau=3.0, u_max=0.05, nu=0.01)
    else:
        rng = np.random.default_rng(11)
        N = nx * ny * nz
        c = {"flags": np.ones((nz, ny, nx), np.int32), "inlets": [], "outlets": [], "nu": 0.004,
             "periodic": (1, 1, 1), "force": (0.0, 0.0, 0.0), "rho": 1 + 0.01 * rng.standard_normal(N),
             "u": 0.03 * rng.standard_normal((3, N))}
    runs = []
    for opt in (capi.LBM_OPT_ROW_STAGING, capi.LBM_OPT_NO_WALL_ROWS):  # the row-staged step has no wall kernel
        s = Solver(shape, turbulence=OmegaLES, storage="f16dev", nu=c["nu"], cles=0.17, periodic=c["periodic"],
                   force=c.get("force", (0, 0, 0)), options=opt)
        s.set_flags(c["flags"])
        s.set_bc()
        s.init_fields(c["rho"], c["u"])
        out = []
        for n in (5, 4):
            s.step(n)
            out.append(s.populations())
        runs.append(out)
        s.close()
    for a, b in zip(*runs):
        assert np.array_equal(a, b)


def _split_case(kind):
    if kind == "channel":  # wall rows, x and z seams
        return (64, 14, 12), cases.channel(64, 14, 12, re_tau=3.0, u_max=0.05, nu=0.01)
    if kind == "box":  # fully periodic: every y/z seam row
        rng = np.random.default_rng(11)
        N = 64 * 8 * 6
        return (64, 8, 6), {"flags": np.ones((6, 8, 64), np.int32), "inlets": [], "outlets": [], "nu": 0.004,
                            "periodic": (1, 1, 1), "force": (0.0, 0.0, 0.0),
                            "rho": 1 + 0.01 * rng.standard_normal(N), "u": 0.03 * rng.standard_normal((3, N))}
    return (40, 16, 14), small_body_case()  # inlet, outlet and body rows beside plain rows


@pytest.mark.parametrize("storage", ["f32", "f16dev"])
@pytest.mark.parametrize("coll,clos", [("cum", "smag"), ("srt", "smag"), ("cum17", "none"), ("comb", "smag"),
                                       ("cum", "mlp"), ("cum", "mlp3")])
@pytest.mark.parametrize("kind", ["channel", "box", "body"])
def test_split_step_is_bit_identical_to_one_launch(built_lib, storage, coll, clos, kind):
    """The default step runs the plain rows (every pair a packed bulk pair off the y/z seams) and the
    remaining rows as two launches; LBM_OPT_ONE_LAUNCH runs one launch over the lattice.  Each slot is
    read and written by one thread within a step, so the populations must agree bit for bit, on odd and
    even steps, for every collision, the learned closure (every step and with a refresh interval of 3)
    and the FP16 stochastic rounding."""
    from lb_gb300 import les
    from lb_gb300.solver import OmegaMLP
    shape, c = _split_case(kind)
    model = None
    turb = CLOS.get(clos, OmegaLES)
    interval = 1
    if clos.startswith("mlp"):
        model = les.MlpModel.load(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                               "lb_gb300", "data", "les_mlp_channel.npz"))
        turb = OmegaMLP
        interval = 3 if clos == "mlp3" else 1
    inlet = InletVelocityEquilibrium if kind == "body" else InletVelocityMovingWall
    runs = []
    # the packed wall-row kernel rounds like the packed path, the one-launch step takes those rows
    # through the per-cell path: compare with it off (its own parity: test_wall_rows_match_oracle)
    for opt in (capi.LBM_OPT_NO_WALL_ROWS, capi.LBM_OPT_ONE_LAUNCH):
        s = Solver(shape, collision=COLL[coll], turbulence=turb, inlet=inlet, storage=storage, nu=c["nu"],
                   cles=0.17, periodic=c.get("periodic", (0, 0, 0)), force=c.get("force", (0, 0, 0)), options=opt,
                   mlp_interval=interval)
        s.set_flags(c["flags"])
        s.set_bc(c.get("inlets", []), c.get("outlets", []))
        if "rho" in c:
            s.init_fields(c["rho"], c["u"])
        else:
            s.init_equilibrium(1.0, (0.04, 0.0, 0.0))
        if model is not None:
            s.load_mlp(model)
        out = []
        for n in (5, 4):
            s.step(n)
            out.append(s.populations())
        runs.append(out)
        s.close()
    for a, b in zip(*runs):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("storage", ["f32", "f16dev"])
@pytest.mark.parametrize("coll,clos", [("cum", "smag"), ("srt", "smag"), ("cum17", "none")])
def test_wall_rows_match_oracle(built_lib, oracle_lib, storage, coll, clos):
    """Rows beside the channel walls take the packed wall kernel (bounce-back links read through the other
    parity's address table).  Against the oracle on a channel whose edge rows are all wall rows: FP32
    within 3e-5 of the FP32 oracle (fp32_parity); FP16 storage within 2e-3 relative L2 of FP64 after 100
    steps; and against the same run with the wall kernel off (LBM_OPT_NO_WALL_ROWS): FP32 within 3e-5."""
    nx, ny, nz = 32, 14, 12
    c = cases.channel(nx, ny, nz, re_tau=3.0, u_max=0.05, nu=0.01)
    g, o = pair((nx, ny, nz), c, coll, clos, storage, 32, force=c["force"])
    _, o64 = pair((nx, ny, nz), c, coll, clos, "f64", 64, force=c["force"])
    init_both(g, o, c)
    assert g.step_launches() == 3  # plain rows, wall rows, the rest (solid rows and z-seam rows)
    o64.init_fields(c["rho"], c["u"])
    if storage == "f32":
        fp32_parity(g, o, o64, 0.05, 100)
        s = Solver((nx, ny, nz), collision=COLL[coll], turbulence=CLOS[clos], storage=storage, nu=c["nu"], cles=0.17,
                   periodic=c["periodic"], force=c["force"], options=capi.LBM_OPT_NO_WALL_ROWS)
        s.set_flags(c["flags"])
        s.set_bc()
        s.init_fields(c["rho"], c["u"])
        s.step(100)
        _, u0 = s.moments()
        _, u1 = g.moments()
        s.close()
        assert np.abs(u1 - u0).max() <= 3e-5 * 0.05
    else:
        g.step(100)
        o64.step(100)
        _, ug = g.moments()
        _, ut = o64.moments()
        fl = c["flags"].reshape(-1) != 0
        assert np.linalg.norm(ug[:, fl] - ut[:, fl]) / np.linalg.norm(ut[:, fl]) < 2e-3


def test_channel_srt_force_fp64(built_lib, oracle_lib):
    nx, ny, nz = 16, 12, 10
    c = cases.channel(nx, ny, nz, re_tau=2.0, u_max=0.04, nu=0.02)  # u_tau = 0.008, F = 1.3e-5
    g, o = pair((nx, ny, nz), c, "srt", "none", "f64", 64, force=c["force"])
    init_both(g, o, c)
    g.step(60)
    o.step(60)
    compare(g, o, 0.04, 1e-12, 1e-12)


def small_body_case(nx=40, ny=16, nz=14):
    body = np.zeros((6, 6, 6), bool)
    body[1:5, 1:5, 1:5] = True
    body[0, 2:4, 2:4] = True
    return cases.body_in_channel(nx, ny, nz, u_in=0.04, rho_out=1.0, nu=0.02, body_flags=body, center=(12, 5, 4))


@pytest.mark.parametrize("coll,clos", [("cum", "smag"), ("srt", "none")])
def test_inlet_outlet_body_fp64(built_lib, oracle_lib, coll, clos):
    c = small_body_case()
    shape = (40, 16, 14)
    g, o = pair(shape, c, coll, clos, "f64", 64, inlet=InletVelocityEquilibrium)
    init_both(g, o, c, 1.0, (0.04, 0, 0))
    for _ in range(4):
        g.step(20)
        o.step(20)
        compare(g, o, 0.04, 1e-12, 1e-12)
    dg = g.reduce()
    do = o.diag()
    assert abs(dg.mass - do.mass) <= 1e-10 * do.mass
    for a in range(3):
        assert abs(dg.drag[a] - do.drag[a]) <= 1e-11 * (abs(do.drag[0]) + 1e-12)
        assert abs(dg.momentum[a] - do.momentum[a]) <= 1e-10 * (abs(do.momentum[0]) + 1e-12)
    assert dg.fluid_cells == do.fluid_cells


def test_inlet_outlet_fp32(built_lib, oracle_lib):
    c = small_body_case()
    shape = (40, 16, 14)
    g, o = pair(shape, c, "cum", "smag", "f32", 32, inlet=InletVelocityEquilibrium)
    _, o64 = pair(shape, c, "cum", "smag", "f64", 64, inlet=InletVelocityEquilibrium)
    init_both(g, o, c, 1.0, (0.04, 0, 0))
    o64.init_equilibrium(1.0, (0.04, 0, 0))
    fp32_parity(g, o, o64, 0.04, 100)


def test_fp16_deviation_storage_tracks_fp64(built_lib, oracle_lib):
    n = 20
    c = cases.cavity(n, u_lid=0.05, re=400.0)
    g, o = pair((n, n, n), c, "cum", "smag", "f16dev", 64)
    init_both(g, o, c)
    g.step(100)
    o.step(100)
    rg, ug = g.moments()
    ro, uo = o.moments()
    fl = c["flags"].reshape(-1) != 0
    rel = np.linalg.norm(ug[:, fl] - uo[:, fl]) / np.linalg.norm(uo[:, fl])
    assert rel < 2e-3, rel
    assert np.abs(rg[fl] - ro[fl]).max() < 2e-3


def test_fp16_stochastic_rounding_keeps_a_weak_body_force(built_lib):
    """Laminar channel driven by twice the force of its initial (steady) profile, so it accelerates by
    ~1.5e-6 per step: the change of a stored population per step (~3e-7) is below half an FP16 step of
    the deviation (~2e-6), so rounding every store to nearest freezes the flow, while stochastic
    rounding (the default) keeps the increments in expectation and tracks FP64.  Tolerance: 2e-3
    relative L2 of the x-z mean velocity profile after 4000 steps."""
    shape = (64, 34, 32)
    nx, ny, nz = shape
    c = cases.channel(*shape, re_tau=8.0, u_max=0.02, amp=0.0, nu=0.01)  # steady at F = 2 nu u_max / h^2
    force = (2.0 * c["force"][0], 0.0, 0.0)
    prof = {}
    for name, storage, opt in (("f64", "f64", 0), ("sr", "f16dev", 0), ("rn", "f16dev", capi.LBM_OPT_F16_ROUND_NEAREST)):
        s = Solver(shape, turbulence=OmegaNo, storage=storage, nu=c["nu"], periodic=c["periodic"], force=force,
                   options=opt)
        s.set_flags(c["flags"])
        s.set_bc()
        s.init_fields(c["rho"], c["u"])
        s.step(4000)
        u = s.moments()[1].reshape(3, nz, ny, nx)
        prof[name] = u[0].mean(axis=(0, 2))[1:-1]
        s.close()
    gain = np.linalg.norm(prof["f64"] - c["u"][0].reshape(nz, ny, nx).mean(axis=(0, 2))[1:-1])
    assert gain > 0.1 * np.linalg.norm(prof["f64"])  # the flow did accelerate
    err = {k: np.linalg.norm(prof[k] - prof["f64"]) / np.linalg.norm(prof["f64"]) for k in ("sr", "rn")}
    assert err["sr"] < 2e-3, err
    assert err["rn"] > 3 * err["sr"], err


def test_populations_fp64_match_oracle(built_lib, oracle_lib):
    c = small_body_case()
    shape = (40, 16, 14)
    g, o = pair(shape, c, "cum", "smag", "f64", 64, inlet=InletVelocityEquilibrium)
    init_both(g, o, c, 1.0, (0.04, 0, 0))
    for n in (7, 8):  # odd and even step counts
        g.step(n)
        o.step(n)
        fg = g.populations()
        fo = o.populations()
        assert np.abs(fg - fo).max() < 1e-13


def test_timeavg_and_error_monitor_match_oracle(built_lib, oracle_lib):
    n = 16
    c = cases.cavity(n, u_lid=0.05, re=200.0)
    g, o = pair((n, n, n), c, "cum", "smag", "f64", 64)
    init_both(g, o, c)
    g.step(10); o.step(10)
    g.timeavg_begin(); o.timeavg_begin()
    g.step(13); o.step(13)
    eg, eo = g.error_evaluation(), o.error()
    assert abs(eg - eo) <= 1e-10 * abs(eo)
    g.step(7); o.step(7)
    g.timeavg_end(); o.timeavg_end()
    rg, ug, uug, cg = g.timeavg_get()
    ro, uo, uuo, co = o.timeavg_get()
    assert cg == co == 20
    assert np.abs(rg - ro).max() < 1e-12 and np.abs(ug - uo).max() < 1e-13 and np.abs(uug - uuo).max() < 1e-14
    eg, eo = g.error_evaluation(), o.error()
    assert abs(eg - eo) <= 1e-10 * abs(eo)


def test_checkpoint_resume_is_bit_identical(built_lib, tmp_path):
    c = small_body_case()
    shape = (40, 16, 14)
    a = Solver(shape, inlet=InletVelocityEquilibrium, turbulence=OmegaLES, storage="f16dev", nu=c["nu"],
               periodic=c["periodic"])
    a.set_flags(c["flags"]); a.set_bc(c["inlets"], c["outlets"]); a.init_equilibrium(1.0, (0.04, 0, 0))
    a.step(11)
    p = tmp_path / "state.lbm"
    a.checkpoint_save(p)
    a.step(9)
    fa = a.populations()
    b = Solver(shape, inlet=InletVelocityEquilibrium, turbulence=OmegaLES, storage="f16dev", nu=c["nu"],
               periodic=c["periodic"])
    b.checkpoint_load(p)
    b.step(9)
    assert np.array_equal(b.populations(), fa)


def test_nonfinite_is_reported(built_lib):
    n = 10
    c = cases.cavity(n)
    s = Solver((n, n, n), storage="f32", nu=c["nu"])
    s.set_flags(c["flags"]); s.set_bc(c["inlets"], [])
    s.init_equilibrium()
    f = s.populations()
    f[5, 5 + n * (5 + n * 5)] = np.nan
    s.set_populations(f)
    d = s.reduce(allow_nonfinite=True)
    assert d.nonfinite >= 1
    with pytest.raises(capi.LbmError) as e:
        s.reduce()
    assert e.value.status == capi.LBM_ERR_NONFINITE


def test_mass_conserved_periodic_box_fp64(built_lib):
    n = 16
    rng = np.random.default_rng(5)
    N = n ** 3
    s = Solver((n, n, n), turbulence=OmegaLES, storage="f64", nu=0.005, periodic=(1, 1, 1))
    s.set_flags(np.ones((n, n, n), np.int32))
    s.set_bc()
    s.init_fields(1 + 0.01 * rng.standard_normal(N), 0.03 * rng.standard_normal((3, N)))
    d0 = s.reduce()
    s.step(50)
    d1 = s.reduce()
    assert abs(d1.mass - d0.mass) < 1e-10 * d0.mass
    assert max(abs(d1.momentum[a] - d0.momentum[a]) for a in range(3)) < 1e-10


GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_gpu_voxelizer_matches_reference_golden(built_lib):
    import ctypes as C
    g = np.load(os.path.join(GOLD, "backward_step_laminar.npz"))
    d = tuple(int(v) for v in g["dims"])
    ref = np.unpackbits(g["packed"])[: d[0] * d[1] * d[2]].reshape(d[2], d[1], d[0]).astype(np.int32)
    dims = np.zeros(3, np.int32)
    bbox = np.zeros(6)
    out = np.zeros(ref.size, np.int32)
    o = np.array([-1.0, -1.0, -1.0])
    L = capi.lib()
    rc = L.lbm_voxelize_off(os.path.join(GOLD, "BackwardStepLaminar.off").encode(), float(g["resolution"]),
                            float(g["additional"]), o.ctypes.data_as(C.POINTER(C.c_double)),
                            out.ctypes.data_as(C.POINTER(C.c_int32)), dims.ctypes.data_as(C.POINTER(C.c_int32)),
                            bbox.ctypes.data_as(C.POINTER(C.c_double)), 0)
    assert rc == 0
    assert tuple(dims) == d
    assert np.array_equal(out.reshape(ref.shape), ref)


def test_gpu_voxelizer_matches_oracle_on_seeded_body(built_lib, oracle_lib):
    import ctypes as C
    v, f = cases.perturbed_icosphere(radius=9.0, subdiv=3, lmax=6, amp=0.15)
    dims = np.zeros(3, np.int32)
    bbox = np.zeros(6)
    L = capi.lib()
    vv = np.ascontiguousarray(v)
    ff = np.ascontiguousarray(f)
    args = (vv.ctypes.data_as(C.POINTER(C.c_double)), len(vv), ff.ctypes.data_as(C.POINTER(C.c_int32)), len(ff),
            1.0, 2.0)
    assert L.lbm_voxelize_mesh(*args, None, dims.ctypes.data_as(C.POINTER(C.c_int32)),
                               bbox.ctypes.data_as(C.POINTER(C.c_double)), 0) == 0
    out = np.zeros(int(dims.prod()), np.int32)
    assert L.lbm_voxelize_mesh(*args, out.ctypes.data_as(C.POINTER(C.c_int32)),
                               dims.ctypes.data_as(C.POINTER(C.c_int32)), bbox.ctypes.data_as(C.POINTER(C.c_double)), 0) == 0
    ref, _ = O.voxelize_mesh(v, f, 1.0, 2.0, (-100.0, -90.0, -80.0))
    assert out.reshape(ref.shape).sum() > 100
    assert np.array_equal(out.reshape(ref.shape), ref)


@pytest.mark.parametrize("storage", ["f64", "f32", "f16dev"])
def test_reductions_are_deterministic_and_match_the_moments(built_lib, storage):
    """lbm_reduce adds per-block FP64 partials in a fixed order: two calls give the same bits, the mass
    equals the FP64 sum of the moments read back per cell, the momentum the sum of rho u, and the error
    monitor repeats its value on an unchanged state."""
    nx, ny, nz = 64, 34, 20
    c = cases.channel(nx, ny, nz, re_tau=3.0, u_max=0.05, nu=0.01, amp=0.05)
    s = Solver((nx, ny, nz), turbulence=OmegaLES, storage=storage, nu=c["nu"], cles=0.17, periodic=c["periodic"],
               force=c["force"])
    s.set_flags(c["flags"])
    s.set_bc()
    s.init_fields(c["rho"], c["u"])
    s.step(7)
    d1, d2 = s.reduce(), s.reduce()
    assert (d1.mass, d1.momentum, d1.max_speed, d1.fluid_cells) == (d2.mass, d2.momentum, d2.max_speed, d2.fluid_cells)
    rho, u = s.moments()
    fl = c["flags"].reshape(-1) != 0
    assert d1.fluid_cells == int(fl.sum())
    assert abs(d1.mass - rho[fl].sum()) <= 1e-12 * rho[fl].sum()
    ref = (rho[fl] * u[0, fl]).sum()
    assert abs(d1.momentum[0] - ref) <= 1e-9 * abs(ref)
    assert abs(d1.max_speed - np.sqrt((u[:, fl] ** 2).sum(axis=0)).max()) <= 1e-6 * d1.max_speed
    e1 = s.error_evaluation()
    e2 = s.error_evaluation()
    assert np.isfinite(e1) and e2 == 0.0
    s.close()


def test_init_from_page_locked_fields_equals_pageable(built_lib):
    """lbm_init_fields reads page-locked host arrays in place (the init kernel's device view of them) and
    copies pageable ones to the device first: both give the same populations bit for bit."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    nx, ny, nz = 32, 18, 10
    c = cases.channel(nx, ny, nz, re_tau=3.0, u_max=0.05, nu=0.01, amp=0.05)
    out = []
    for pinned in (False, True):
        rho, u = c["rho"].astype(np.float64), c["u"].astype(np.float64)
        if pinned:
            tr = torch.empty(rho.size, dtype=torch.float64, pin_memory=True)
            tu = torch.empty(u.size, dtype=torch.float64, pin_memory=True)
            tr.numpy()[...] = rho.reshape(-1)
            tu.numpy()[...] = u.reshape(-1)
            rho, u = tr.numpy().reshape(c["rho"].shape), tu.numpy().reshape(c["u"].shape)
        s = Solver((nx, ny, nz), turbulence=OmegaLES, storage="f32", nu=c["nu"], cles=0.17, periodic=c["periodic"],
                   force=c["force"])
        s.set_flags(c["flags"])
        s.set_bc()
        s.init_fields(rho, u)
        out.append(s.populations())
        s.close()
    assert np.array_equal(out[0], out[1])
