"""GPU kernels (through the C ABI) against the oracle on the remaining boundary policies: InletVelocityZouHe,
the neighbour-equilibrium outlets with and without the sponge, OutletDensityEquilibrium and
BounceSymmetryHalf.

Tolerances (stated per test): FP64 GPU vs FP64 oracle <= 1e-12 on rho and on u relative to the inlet
speed; FP32 GPU within 3e-5 of the FP32 oracle; FP16-deviation storage within 2e-3 relative L2 of the
FP64 oracle after 100 steps; a half channel with a symmetry plane equal to the mirrored full channel to
1e-12 (FP64) on the GPU as in the oracle.
"""
import numpy as np
import pytest

from lb_gb300 import capi, cases
from lb_gb300.solver import (CollisionCumD3Q27Turbulent2015, InletVelocityEquilibrium, InletVelocityMovingWall,
                             InletVelocityZouHe, OmegaLES, OutletDensityEquilibrium, OutletDensityInterpolated,
                             OutletNeighbourEquilibrium, OutletNeighbourEquilibriumOmega,
                             OutletNeighbourEquilibriumOmegaRF, Solver)
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DUMP = (0.0, 0.05)  # omegaDumpingLow / High of the reference's main.cu:137-138


def duct_pair(shape, inlet, outlet, storage, prec):
    c = cases.duct(*shape)
    g = Solver(shape, collision=CollisionCumD3Q27Turbulent2015, turbulence=OmegaLES, inlet=inlet, outlet=outlet,
               storage=storage, nu=c["nu"], cles=0.17, periodic=c["periodic"], omega_dumping=DUMP)
    g.set_flags(c["flags"])
    g.set_bc(c["inlets"], c["outlets"])
    g.init_fields(c["rho"], c["u"])
    cfg = capi.make_config(*shape, periodic=c["periodic"], collision=capi.LBM_COLLISION_CUMULANT2015,
                           closure=capi.LBM_CLOSURE_SMAGORINSKY, inlet_kind=inlet.code, nu=c["nu"], cles=0.17,
                           outlet_kind=outlet.code, omega_dumping=DUMP)
    o = O.OracleSim(cfg, prec)
    o.set_flags(c["flags"])
    o.set_bc(c["inlets"], c["outlets"])
    o.init_fields(c["rho"], c["u"])
    return g, o, c


def max_diff(g, o):
    rg, ug = g.moments()
    ro, uo = o.moments()
    return np.abs(rg - ro).max(), np.abs(ug - uo).max()


@pytest.mark.parametrize("inlet,outlet", [
    (InletVelocityZouHe, OutletNeighbourEquilibrium),
    (InletVelocityZouHe, OutletNeighbourEquilibriumOmega),
    (InletVelocityEquilibrium, OutletNeighbourEquilibriumOmegaRF),
    (InletVelocityMovingWall, OutletDensityEquilibrium),
    (InletVelocityZouHe, OutletDensityInterpolated),
])
def test_duct_boundaries_fp64_match_oracle(built_lib, oracle_lib, inlet, outlet):
    """A perturbed duct (seeded noise of 30 % of the inlet speed, so some outlet nodes see backflow and the
    RF density correction acts); the sponge covers x = 21..23."""
    shape = (24, 10, 8)
    g, o, c = duct_pair(shape, inlet, outlet, "f64", 64)
    for _ in range(3):
        g.step(20)
        o.step(20)
        dr, du = max_diff(g, o)
        assert dr <= 1e-12 and du <= 1e-12 * 0.04, (dr, du)


def test_duct_neighbour_equilibrium_fp32(built_lib, oracle_lib):
    """FP32 storage, packed pairs in the bulk and the per-cell path in the sponge and on the boundary
    planes: within 3e-5 of the inlet speed of the FP32 oracle after 100 steps."""
    shape = (24, 10, 8)
    g, o, c = duct_pair(shape, InletVelocityZouHe, OutletNeighbourEquilibriumOmega, "f32", 32)
    g.step(100)
    o.step(100)
    dr, du = max_diff(g, o)
    assert dr <= 3e-5 and du <= 3e-5 * 0.04, (dr, du)


def test_duct_neighbour_equilibrium_f16dev(built_lib, oracle_lib):
    shape = (24, 10, 8)
    g, o, c = duct_pair(shape, InletVelocityZouHe, OutletNeighbourEquilibriumOmegaRF, "f16dev", 64)
    g.step(100)
    o.step(100)
    _, ug = g.moments()
    _, uo = o.moments()
    assert np.linalg.norm(ug - uo) / np.linalg.norm(uo) < 2e-3


def run_symmetric(storage, prec=None):
    half, full = cases.symmetric_channel(16, 6, 8)
    out = []
    for c, shape in ((half, (16, 8, 8)), (full, (16, 14, 8))):
        g = Solver(shape, turbulence=OmegaLES, storage=storage, nu=c["nu"], cles=0.17, periodic=c["periodic"],
                   force=c["force"])
        g.set_flags(c["flags"])
        g.set_bc()
        if "symmetry" in c:
            g.set_symmetry(c["symmetry"])
        g.init_fields(c["rho"], c["u"])
        o = None
        if prec:
            cfg = capi.make_config(*shape, periodic=c["periodic"], closure=capi.LBM_CLOSURE_SMAGORINSKY, nu=c["nu"],
                                   cles=0.17, force=c["force"])
            o = O.OracleSim(cfg, prec)
            o.set_flags(c["flags"])
            o.set_bc()
            if "symmetry" in c:
                o.set_symmetry(c["symmetry"])
            o.init_fields(c["rho"], c["u"])
        out.append((g, o, shape))
    return out


def test_symmetry_plane_fp64_matches_oracle_and_full_channel(built_lib, oracle_lib):
    """BounceSymmetryHalf on the GPU: the half channel equals the oracle's (1e-12) and its rows 0..6 equal
    the GPU's mirrored full channel (1e-12), over odd and even steps."""
    (gh, oh, sh), (gf, _, sf) = run_symmetric("f64", 64)
    for n in (7, 20, 33):
        gh.step(n)
        oh.step(n)
        gf.step(n)
        dr, du = max_diff(gh, oh)
        assert dr <= 1e-12 and du <= 1e-12 * 0.05, (dr, du)
        _, uh = gh.moments()
        _, uf = gf.moments()
        uh = uh.reshape(3, sh[2], sh[1], sh[0])[:, :, :7, :]
        uf = uf.reshape(3, sf[2], sf[1], sf[0])[:, :, :7, :]
        assert np.abs(uh - uf).max() <= 1e-12 * 0.05


@pytest.mark.parametrize("storage", ["f32", "f16dev"])
def test_symmetry_plane_packed_storage(built_lib, oracle_lib, storage):
    """FP32 within 3e-5 of the FP32 oracle; FP16-deviation within 2e-3 relative L2 of the FP64 oracle
    (100 steps)."""
    (gh, oh, sh), _ = run_symmetric(storage, 32 if storage == "f32" else 64)
    gh.step(100)
    oh.step(100)
    _, ug = gh.moments()
    _, uo = oh.moments()
    if storage == "f32":
        assert np.abs(ug - uo).max() <= 3e-5 * 0.05
    else:
        assert np.linalg.norm(ug - uo) / np.linalg.norm(uo) < 2e-3


def test_checkpoint_resume_with_side_tables_is_bit_identical(built_lib, tmp_path):
    """The neighbour-equilibrium outlet keeps moments between steps and the symmetry records live in
    the checkpoint: a resumed run continues bit for bit."""
    shape = (24, 10, 8)
    c = cases.duct(*shape)

    def make():
        s = Solver(shape, turbulence=OmegaLES, inlet=InletVelocityZouHe, outlet=OutletNeighbourEquilibriumOmega,
                   storage="f16dev", nu=c["nu"], cles=0.17, periodic=c["periodic"], omega_dumping=DUMP)
        return s

    a = make()
    a.set_flags(c["flags"]); a.set_bc(c["inlets"], c["outlets"]); a.init_fields(c["rho"], c["u"])
    a.step(11)
    p = tmp_path / "state.lbm"
    a.checkpoint_save(p)
    a.step(9)
    fa = a.populations()
    b = make()
    b.checkpoint_load(p)
    b.step(9)
    assert np.array_equal(b.populations(), fa)

    half, _ = cases.symmetric_channel(16, 6, 8)
    s1 = Solver((16, 8, 8), turbulence=OmegaLES, storage="f32", nu=half["nu"], periodic=half["periodic"],
                force=half["force"])
    s1.set_flags(half["flags"]); s1.set_bc(); s1.set_symmetry(half["symmetry"]); s1.init_fields(half["rho"], half["u"])
    s1.step(6)
    s1.checkpoint_save(p)
    s1.step(5)
    f1 = s1.populations()
    s2 = Solver((16, 8, 8), turbulence=OmegaLES, storage="f32", nu=half["nu"], periodic=half["periodic"],
                force=half["force"])
    s2.checkpoint_load(p)
    s2.step(5)
    assert np.array_equal(s2.populations(), f1)


def test_unsupported_boundary_setups_are_rejected(built_lib):
    """Set-up checks (host side, before any kernel): symmetry normals other than +-y, a symmetry plane
    without a solid row across it, a neighbour-equilibrium outlet whose upstream cell is not fluid."""
    half, _ = cases.symmetric_channel(16, 6, 8)

    def sym_status(records):
        s = Solver((16, 8, 8), turbulence=OmegaLES, storage="f32", nu=half["nu"], periodic=half["periodic"])
        s.set_flags(half["flags"])
        s.set_bc()
        s.set_symmetry(records)
        with pytest.raises(capi.LbmError) as e:
            s.init_fields(half["rho"], half["u"])
        s.close()
        return e.value.status

    recs = half["symmetry"]
    assert sym_status([capi.make_symmetry(r.vertex.x, r.vertex.y, r.vertex.z, (1, 0, 0), 1) for r in recs]) == \
        capi.LBM_ERR_UNSUPPORTED
    # normal -y: the row "across" is the fluid row below the plane
    assert sym_status([capi.make_symmetry(r.vertex.x, r.vertex.y, r.vertex.z, (0, -1, 0), 1) for r in recs]) == \
        capi.LBM_ERR_UNSUPPORTED
    c = cases.duct(24, 10, 8)
    f = c["flags"].copy()
    f[3, 4, 22] = 0  # a solid cell upstream of the outlet plane
    s = Solver((24, 10, 8), turbulence=OmegaLES, inlet=InletVelocityZouHe, outlet=OutletNeighbourEquilibrium,
               storage="f32", nu=c["nu"], periodic=c["periodic"])
    s.set_flags(f)
    s.set_bc(c["inlets"], c["outlets"])
    with pytest.raises(capi.LbmError) as e:
        s.init_fields(c["rho"], c["u"])
    assert e.value.status == capi.LBM_ERR_UNSUPPORTED
