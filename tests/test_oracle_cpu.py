"""CPU tests of the oracle: pinned against the reference's golden voxel matrix and checked on
known-answer properties of the solver hooks."""
import os

import numpy as np
import pytest

from lb_gb300 import capi, cases
from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def golden():
    g = np.load(os.path.join(GOLD, "backward_step_laminar.npz"))
    d = tuple(int(v) for v in g["dims"])
    flags = np.unpackbits(g["packed"])[: d[0] * d[1] * d[2]].reshape(d[2], d[1], d[0]).astype(np.int32)
    return g, d, flags


def test_golden_fixture_counts():
    g, d, flags = golden()
    assert d == (377, 52, 52)
    assert int(flags.sum()) == 843750 == int(g["count_inside"])


def test_oracle_voxelizer_matches_reference_golden(oracle_lib):
    g, d, ref = golden()
    flags, bbox = O.voxelize_off(os.path.join(GOLD, "BackwardStepLaminar.off"), float(g["resolution"]),
                                 float(g["additional"]), (-1.0, -1.0, -1.0))
    assert flags.shape == ref.shape
    assert np.array_equal(flags, ref)
    assert np.allclose(bbox[:3], g["bbmin"]) and np.allclose(bbox[3:], g["bbmax"])


def test_oracle_voxelizer_outside_point_independent(oracle_lib):
    # a closed mesh: the parity must not depend on the outside reference point
    g, d, ref = golden()
    flags, _ = O.voxelize_off(os.path.join(GOLD, "BackwardStepLaminar.off"), float(g["resolution"]),
                              float(g["additional"]), (-37.0, 251.0, -13.0))
    assert np.array_equal(flags, ref)


W = np.array([8 / 27] + [2 / 27] * 6 + [1 / 54] * 12 + [1 / 216] * 8)
CV = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 0, -1], [0, 0, 1], [0, -1, 0], [0, 1, 0], [1, 0, -1],
               [-1, 0, 1], [1, 0, 1], [-1, 0, -1], [-1, -1, 0], [1, 1, 0], [0, 1, -1], [0, -1, 1], [-1, 1, 0],
               [1, -1, 0], [0, 1, 1], [0, -1, -1], [-1, 1, -1], [1, -1, 1], [-1, -1, 1], [1, 1, -1], [1, -1, -1],
               [-1, 1, 1], [-1, -1, -1], [1, 1, 1]])


def feq(r, u):
    cu = CV @ u
    return W * r * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * u @ u)


@pytest.mark.parametrize("coll", [capi.LBM_COLLISION_SRT, capi.LBM_COLLISION_CUMULANT2015,
                                  capi.LBM_COLLISION_CUMULANT2017, capi.LBM_COLLISION_CUMULANT_COMBINED])
def test_collision_conserves_mass_and_momentum(oracle_lib, coll):
    rng = np.random.default_rng(1)
    for _ in range(5):
        u = rng.uniform(-0.05, 0.05, 3)
        f = feq(1 + rng.uniform(-0.02, 0.02), u) * (1 + 0.02 * rng.standard_normal(27))
        r = f.sum()
        uu = CV.T @ f / r
        out = O.collide_cell(f, r, uu, rng.uniform(0.6, 1.9), coll, flag=3)  # combined: its 2017 branch
        assert abs(out.sum() - f.sum()) < 1e-14
        assert np.abs(CV.T @ out - CV.T @ f).max() < 1e-14


def test_srt_equilibrium_is_fixed_point(oracle_lib):
    u = np.array([0.03, -0.02, 0.01])
    f = feq(1.03, u)
    assert np.abs(O.collide_cell(f, 1.03, u, 1.3, capi.LBM_COLLISION_SRT) - f).max() < 1e-15


def test_cumulant_relaxes_shear_stress(oracle_lib):
    # omega = 1 sets the off-diagonal second cumulant to zero: <c_x c_y (f*)> = rho u_x u_y
    rng = np.random.default_rng(3)
    u = np.array([0.02, 0.01, -0.015])
    f = feq(1.0, u) * (1 + 0.05 * rng.standard_normal(27))
    r = f.sum()
    uu = CV.T @ f / r
    out = O.collide_cell(f, r, uu, 1.0, capi.LBM_COLLISION_CUMULANT2015)
    pxy = (CV[:, 0] * CV[:, 1]) @ out
    assert abs(pxy - r * uu[0] * uu[1]) < 1e-14


def test_wall_pass_matches_oracle_and_numpy(oracle_lib, built_lib):
    rng = np.random.default_rng(0)
    f = (rng.random((9, 11, 13)) > 0.3).astype(np.int32)
    a = O.wall_pass(f.copy())
    b = cases.wall_pass_numpy(f)
    c = cases.wall_pass(f.copy())
    assert np.array_equal(a, b) and np.array_equal(a, c)


def _box_sim(n, flags, periodic, **kw):
    cfg = capi.make_config(*n, periodic=periodic, **kw)
    s = O.OracleSim(cfg, 64)
    s.set_flags(flags)
    return s


def test_ghost_plane_periodic_equals_index_wrap(oracle_lib):
    """Periodic.h ghost planes (planes 1 and L+1 mirror each other, perIdx pointing across) on a
    box wrapped in y, z == native wrap in x over the L interior planes."""
    L, ny, nz = 10, 6, 5
    rng = np.random.default_rng(7)
    N = L * ny * nz
    rho = 1 + 0.01 * rng.standard_normal(N)
    u = 0.03 * rng.standard_normal((3, N))
    # native wrap: planes 0..L-1
    a = _box_sim((L, ny, nz), np.ones((nz, ny, L), np.int32), (1, 1, 1), nu=0.02,
                 collision=capi.LBM_COLLISION_CUMULANT2015, closure=capi.LBM_CLOSURE_SMAGORINSKY)
    a.init_fields(rho, u)
    # ghost form: X = L + 3 planes: solid 0, periodic 1 (copy of plane L+1... see below), interior, solid last
    X = L + 3
    fl = np.ones((nz, ny, X), np.int32)
    fl[:, :, 0] = 0
    fl[:, :, -1] = 0
    fl[:, :, 1] = -3
    fl[:, :, L + 1] = -3
    # plane p in the ghost lattice holds native plane (p-1) mod L; plane L+1 duplicates plane 1 (native 0)
    rho_g = np.ones((nz, ny, X))
    u_g = np.zeros((3, nz, ny, X))
    r3 = rho.reshape(nz, ny, L)
    u3 = u.reshape(3, nz, ny, L)
    for p in range(1, L + 2):
        rho_g[:, :, p] = r3[:, :, (p - 1) % L]
        u_g[:, :, :, p] = u3[:, :, :, (p - 1) % L]
    b = _box_sim((X, ny, nz), fl, (0, 1, 1), nu=0.02, collision=capi.LBM_COLLISION_CUMULANT2015,
                 closure=capi.LBM_CLOSURE_SMAGORINSKY)
    recs = []
    for k in range(nz):
        for j in range(ny):
            recs.append([1, j, k, -1, 0, 0, L + 1, 0])    # plane 1, normal -x, copies from plane L+1
            recs.append([L + 1, j, k, 1, 0, 0, 1, 0])     # plane L+1, normal +x, copies from plane 1
    b.set_periodic_list(recs)
    b.init_fields(rho_g.reshape(-1), u_g.reshape(3, -1))
    for _ in range(6):
        a.step(1)
        b.step(1)
        ra, ua = a.moments()
        rb, ub = b.moments()
        ra = ra.reshape(nz, ny, L)
        rb = rb.reshape(nz, ny, X)[:, :, 1:L + 1]
        assert np.abs(ra - rb).max() < 1e-13
        assert np.abs(ua.reshape(3, nz, ny, L) - ub.reshape(3, nz, ny, X)[:, :, :, 1:L + 1]).max() < 1e-13


def test_cavity_mass_conserved_and_lid_drives_flow(oracle_lib):
    c = cases.cavity(12, u_lid=0.05, re=100.0)
    cfg = capi.make_config(12, 12, 12, collision=capi.LBM_COLLISION_CUMULANT2015, nu=c["nu"])
    s = O.OracleSim(cfg, 64)
    s.set_flags(c["flags"])
    s.set_bc(c["inlets"], [])
    s.init_equilibrium(1.0, (0, 0, 0))
    m0 = s.diag().mass
    s.step(50)
    d = s.diag()
    rho, u = s.moments()
    ux = u[0].reshape(12, 12, 12)
    assert d.nonfinite == 0
    assert ux[6, 10, 6] > 0.005          # flow under the lid moves with it
    assert abs(d.mass - m0) / m0 < 1e-3  # moving-wall nodes exchange little mass


def feq_factorised(r, u):
    """The product-form D3Q27 equilibrium: every cumulant above second order is zero."""
    def phi(c, a):
        return np.where(c == 0, 2.0 / 3.0 - a * a, 0.5 * (1.0 / 3.0 + a * a + c * a))
    return r * phi(CV[:, 0], u[0]) * phi(CV[:, 1], u[1]) * phi(CV[:, 2], u[2])


@pytest.mark.parametrize("coll", [capi.LBM_COLLISION_CUMULANT2015, capi.LBM_COLLISION_CUMULANT2017])
def test_cumulant_equilibrium_is_fixed_point(oracle_lib, coll):
    """CollisionCumD3Q27Turbulent2015/2017: the cumulant equilibrium of a moving fluid is left unchanged.
    The 2017 reference's bulk term (-(rho - 1) in Dxu, CollisionCumD3Q27Turbulent2017.h:295) breaks this:
    it reads a velocity gradient of -1/(2 rho) into a fluid at rest in its own frame."""
    u = np.array([0.04, -0.03, 0.02])
    f = feq_factorised(1.02, u)
    out = O.collide_cell(f, f.sum(), CV.T @ f / f.sum(), 1.7, coll)
    assert np.abs(out - f).max() < 1e-15
    if coll == capi.LBM_COLLISION_CUMULANT2017:
        ref = O.collide_cell(f, f.sum(), CV.T @ f / f.sum(), 1.7, coll, ref_compat=True)
        assert np.abs(ref - f).max() > 1e-5


def _permute_axes(f, perm):
    """Populations of the same state with axes relabelled: new axis a is old axis perm[a]."""
    idx = {tuple(c): v for v, c in enumerate(CV)}
    g = np.empty(27)
    for v, c in enumerate(CV):
        g[idx[tuple(c[list(perm)])]] = f[v]
    return g


def test_cumulant2017_commutes_with_axis_relabelling(oracle_lib):
    """The corrected 2017 operator is isotropic: relabelling x, y, z before or after the collision gives
    the same populations, for a rotation and for the three transpositions.  Two reference lines break
    this and ref_compat reproduces them: the limiters of the 210/012 pair read C120 +- C102
    (CollisionCumD3Q27Turbulent2017.h:256-266), and eq. 44 pairs C220 + C202 - 2 C022 with
    Dxu + Dyv - 2 Dzw (:351), whose axis image is Dyv + Dzw - 2 Dxu."""
    rng = np.random.default_rng(5)
    u = np.array([0.03, -0.01, 0.02])
    f = feq(1.0, u) * (1 + 0.05 * rng.standard_normal(27))
    r = f.sum()
    uu = CV.T @ f / r
    for perm in ((1, 2, 0), (1, 0, 2), (0, 2, 1), (2, 1, 0)):
        fp = _permute_axes(f, perm)
        up = uu[list(perm)]
        for ref, expect_equal in ((False, True), (True, False)):
            a = _permute_axes(O.collide_cell(f, r, uu, 1.8, capi.LBM_COLLISION_CUMULANT2017, ref_compat=ref), perm)
            b = O.collide_cell(fp, r, up, 1.8, capi.LBM_COLLISION_CUMULANT2017, ref_compat=ref)
            assert (np.abs(a - b).max() < 1e-15) == expect_equal, (perm, ref, np.abs(a - b).max())


def test_combined_collision_picks_the_operator_by_flag(oracle_lib):
    """CollisionCumD3Q27TurbulentCombined: cells of flag 1 take the 2015 operator, every other nonzero
    flag (wall-pass counts, boundary nodes) the 2017 one (CollisionCumD3Q27TurbulentCombined.h:1066-1078).
    Its 2017 copy differs from the 2017 header in one reference line only, the bulk term of Dxu
    (:295, - -(-1 - rho) against - (-1 + rho)), so the two agree when corrected and differ with
    ref_compat."""
    rng = np.random.default_rng(9)
    u = np.array([0.02, 0.03, -0.01])
    f = feq(1.01, u) * (1 + 0.03 * rng.standard_normal(27))
    r = f.sum()
    uu = CV.T @ f / r
    comb = capi.LBM_COLLISION_CUMULANT_COMBINED
    c15 = O.collide_cell(f, r, uu, 1.9, capi.LBM_COLLISION_CUMULANT2015)
    c17 = O.collide_cell(f, r, uu, 1.9, capi.LBM_COLLISION_CUMULANT2017)
    assert np.abs(c15 - c17).max() > 1e-8
    assert np.array_equal(O.collide_cell(f, r, uu, 1.9, comb, flag=1), c15)
    for flag in (2, 7, -1, -2, -3):
        assert np.array_equal(O.collide_cell(f, r, uu, 1.9, comb, flag=flag), c17)
    ref17 = O.collide_cell(f, r, uu, 1.9, capi.LBM_COLLISION_CUMULANT2017, ref_compat=True)
    refc = O.collide_cell(f, r, uu, 1.9, comb, ref_compat=True, flag=7)
    assert np.abs(refc - ref17).max() > 1e-6


def test_wall_policies_differ_only_in_the_reference_selection(oracle_lib):
    """BounceBackWallHalf bounces back on the wall list (flag > 2 in the reference,
    geometryMesherBoundary.h:459), BounceBackWallHalfMesh on the cells of flag exactly 2
    (BounceBackWallHalfMesh.h:38); corrected, both take every fluid cell with a solid neighbour."""
    from lb_gb300 import cases
    f0 = np.ones((10, 10, 10), np.int32)
    f0[[0, -1], :, :] = 0
    f0[:, [0, -1], :] = 0
    f0[:, :, [0, -1]] = 0
    f0[5, 5, 5] = 0  # an isolated solid cell: its 26 neighbours have flag 2
    flags = cases.wall_pass_numpy(f0)
    assert np.sum(flags == 2) == 26
    cfg = capi.make_config(10, 10, 10, nu=0.05)
    sizes = {}
    for ref in (False, True):
        for mesh in (0, 1):
            o = O.OracleSim(cfg, 64, ref_compat=ref)
            o.set_flags(flags)
            o.set_wall_policy(mesh)
            sizes[(ref, mesh)] = o.wall_list_size()
    f = flags.reshape(-1)
    assert sizes[(False, 0)] == sizes[(False, 1)] == int(np.sum(f > 1))
    assert sizes[(True, 0)] == int(np.sum(f > 2)) and sizes[(True, 1)] == int(np.sum(f == 2))
