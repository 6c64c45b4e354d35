"""The oracle's restatement of the remaining boundary policies, checked by known answers on the CPU:
BounceSymmetryHalf (a half channel with a symmetry plane is the full channel), the
OutletNeighbourEquilibriumOmega sponge (its relaxation-rate ramp), InletVelocityZouHe and the outlet
variants (a uniform stream is a fixed point).  The reference defects reproduced under ref_compat must
break the known answers where they apply."""
import numpy as np
import pytest

from lb_gb300 import capi, cases
from oracle import oracle as O

OUTLETS = [capi.LBM_OUTLET_DENSITY_INTERPOLATED, capi.LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM,
           capi.LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA, capi.LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA_RF,
           capi.LBM_OUTLET_DENSITY_EQUILIBRIUM]


def run_symmetric(ref_compat, steps=60):
    half, full = cases.symmetric_channel(8, 5, 6)
    out = []
    for c, shape in ((half, (8, 7, 6)), (full, (8, 12, 6))):
        cfg = capi.make_config(*shape, periodic=c["periodic"], collision=capi.LBM_COLLISION_CUMULANT2015,
                               closure=capi.LBM_CLOSURE_SMAGORINSKY, nu=c["nu"], cles=0.17, force=c["force"])
        o = O.OracleSim(cfg, 64, ref_compat=ref_compat)
        o.set_flags(c["flags"])
        o.set_bc()
        if "symmetry" in c:
            o.set_symmetry(c["symmetry"])
        o.init_fields(c["rho"], c["u"])
        o.step(steps)
        _, u = o.moments()
        out.append(u.reshape(3, shape[2], shape[1], shape[0]))
    return out


def test_symmetry_plane_reproduces_the_full_channel(oracle_lib):
    """BounceSymmetryHalf.h:84-131 at y = 5 (normal +y): the half channel's rows 0..5 equal the rows of
    the channel twice as high whose initial field is mirrored about y = 5.5, because the populations a
    mirror image sends across the plane are exactly the reflected ones.  The reference's c_sym_y table
    (D3Q27.h:162-190) maps seven directions to the wrong mirror, and breaks this."""
    uh, uf = run_symmetric(False)
    assert np.abs(uh[:, :, :6, :] - uf[:, :, :6, :]).max() < 1e-13
    assert np.abs(uh[0]).max() > 0.01  # the flow is not trivial
    uh_ref, uf_ref = run_symmetric(True)
    assert np.abs(uh_ref[:, :, :6, :] - uf_ref[:, :, :6, :]).max() > 1e-6


def test_outlet_sponge_lowers_omega_linearly(oracle_lib):
    """OutletNeighbourEquilibriumOmega.h:18-79: over the last ceil(0.1 nx) planes (nx = 24: x = 21..23)
    omega = 1/tau - (high - low) / 3 * (x - 21); elsewhere 1/tau (OmegaNo)."""
    c = cases.duct(24, 6, 5)
    cfg = capi.make_config(24, 6, 5, periodic=c["periodic"], collision=capi.LBM_COLLISION_CUMULANT2015,
                           closure=capi.LBM_CLOSURE_NONE, inlet_kind=capi.LBM_INLET_ZOU_HE, nu=c["nu"],
                           outlet_kind=capi.LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA, omega_dumping=(0.0, 0.05))
    o = O.OracleSim(cfg, 64)
    o.set_flags(c["flags"])
    o.set_bc(c["inlets"], c["outlets"])
    o.init_fields(c["rho"], c["u"])
    o.step(1)
    om = o.omega().reshape(5, 6, 24)
    w0 = 1.0 / (3 * c["nu"] + 0.5)
    expect = np.full(24, w0)
    expect[21:] -= 0.05 / 3 * np.arange(3)
    assert np.allclose(om, expect[None, None, :], rtol=0, atol=1e-15)


@pytest.mark.parametrize("outlet", OUTLETS)
@pytest.mark.parametrize("inlet", [capi.LBM_INLET_ZOU_HE, capi.LBM_INLET_MOVING_WALL])
def test_uniform_stream_is_kept(oracle_lib, inlet, outlet):
    """A uniform stream at the inlet velocity and the outlet density is an equilibrium of every pass:
    the inlets (InletVelocityZouHe.h:85-97, InletVelocityMovingWall.h:40-53), each outlet, and the
    sponge (equilibrium is a fixed point for any relaxation rate).  SRT collision: its fixed point is the
    polynomial equilibrium the state starts from.  u0 = 5/128 is exact in the records' FP32 velocity."""
    nx, ny, nz, u0 = 16, 5, 4, 0.0390625
    c = cases.duct(nx, ny, nz, u_in=u0, amp=0.0)
    cfg = capi.make_config(nx, ny, nz, periodic=c["periodic"], collision=capi.LBM_COLLISION_SRT,
                           closure=capi.LBM_CLOSURE_SMAGORINSKY, inlet_kind=inlet, nu=c["nu"], cles=0.17,
                           outlet_kind=outlet, omega_dumping=(0.0, 0.05))
    o = O.OracleSim(cfg, 64)
    o.set_flags(c["flags"])
    o.set_bc(c["inlets"], c["outlets"])
    o.init_fields(np.ones(nx * ny * nz), c["u"])
    o.step(20)
    rho, u = o.moments()
    assert np.abs(rho - 1.0).max() < 1e-13
    assert np.abs(u[0] - u0).max() < 1e-13 and np.abs(u[1:]).max() < 1e-13


def test_density_equilibrium_outlet_defect_breaks_the_uniform_stream(oracle_lib):
    """OutletDensityEquilibrium.h:66 writes f_eq of the outgoing direction v into slot c_rev[v]; with a
    moving fluid that is not the equilibrium of the entering direction."""
    nx, ny, nz, u0 = 16, 5, 4, 0.0390625
    c = cases.duct(nx, ny, nz, u_in=u0, amp=0.0)
    cfg = capi.make_config(nx, ny, nz, periodic=c["periodic"], collision=capi.LBM_COLLISION_SRT,
                           inlet_kind=capi.LBM_INLET_ZOU_HE, nu=c["nu"], outlet_kind=capi.LBM_OUTLET_DENSITY_EQUILIBRIUM)
    o = O.OracleSim(cfg, 64, ref_compat=True)
    o.set_flags(c["flags"])
    o.set_bc(c["inlets"], c["outlets"])
    o.init_fields(np.ones(nx * ny * nz), c["u"])
    o.step(5)
    _, u = o.moments()
    assert np.abs(u[0] - u0).max() > 1e-4


def test_neighbour_equilibrium_outlet_matches_its_definition(oracle_lib):
    """One step of OutletNeighbourEquilibrium (:93-125) on a perturbed duct: each entering link of an
    outlet node equals f_eq_v(u(x), rho_b) + f_eq_v(x + c_v) - f_v(x + c_v), with u, rho the moments
    before the step and f(x + c_v) the neighbour's populations after streaming (the outlet node's own
    post-collision f*_v).  With the non-equilibrium part's sign reversed, f_v + f*_v feedback makes the
    same duct diverge (density NaN within 50 steps): the reference's sign is the stable one."""
    nx, ny, nz = 12, 4, 4
    c = cases.duct(nx, ny, nz)
    cfg = capi.make_config(nx, ny, nz, periodic=c["periodic"], inlet_kind=capi.LBM_INLET_ZOU_HE, nu=c["nu"],
                           outlet_kind=capi.LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM)
    o = O.OracleSim(cfg, 64)
    o.set_flags(c["flags"])
    o.set_bc(c["inlets"], c["outlets"])
    o.init_fields(c["rho"], c["u"])
    o.step(3)
    rho0, u0 = o.moments()
    rho0, u0 = rho0.reshape(nz, ny, nx), u0.reshape(3, nz, ny, nx)
    o.step(1)
    f = o.populations().reshape(27, nz, ny, nx)
    w = np.array([8 / 27] + [2 / 27] * 6 + [1 / 54] * 12 + [1 / 216] * 8)
    CV = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 0, -1], [0, 0, 1], [0, -1, 0], [0, 1, 0], [1, 0, -1],
                   [-1, 0, 1], [1, 0, 1], [-1, 0, -1], [-1, -1, 0], [1, 1, 0], [0, 1, -1], [0, -1, 1], [-1, 1, 0],
                   [1, -1, 0], [0, 1, 1], [0, -1, -1], [-1, 1, -1], [1, -1, 1], [-1, -1, 1], [1, 1, -1],
                   [1, -1, -1], [-1, 1, 1], [-1, -1, -1], [1, 1, 1]])

    def feq(v, r, u):
        cu = CV[v] @ u
        return w[v] * r * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * u @ u)

    x = nx - 1
    worst = 0.0
    for k in range(nz):
        for j in range(ny):
            for v in range(27):
                if CV[v][0] != -1:
                    continue
                a, b, g = x - 1, (j + CV[v][1]) % ny, (k + CV[v][2]) % nz
                fb = feq(v, 1.0, u0[:, k, j, x])
                worst = max(worst, abs(f[v, k, j, x] - (fb + feq(v, rho0[g, b, a], u0[:, g, b, a]) - f[v, g, b, a])))
    assert worst < 1e-15


def test_neighbour_equilibrium_outlet_carries_the_stream(oracle_lib):
    """300 steps of the perturbed duct with a Zou/He inlet and the sponge outlet: the density settles
    within 1e-3 of the outlet's and the mean velocity next to the outlet within 1 % of the inlet's."""
    nx, ny, nz = 24, 10, 8
    c = cases.duct(nx, ny, nz)
    cfg = capi.make_config(nx, ny, nz, periodic=c["periodic"], closure=capi.LBM_CLOSURE_SMAGORINSKY, cles=0.17,
                           inlet_kind=capi.LBM_INLET_ZOU_HE, nu=c["nu"],
                           outlet_kind=capi.LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA, omega_dumping=(0.0, 0.05))
    o = O.OracleSim(cfg, 64)
    o.set_flags(c["flags"])
    o.set_bc(c["inlets"], c["outlets"])
    o.init_fields(c["rho"], c["u"])
    o.step(300)
    r, u = o.moments()
    r, u = r.reshape(nz, ny, nx), u.reshape(3, nz, ny, nx)
    assert np.abs(r[:, :, 1:-1] - 1.0).max() < 1e-3
    assert abs(u[0, :, :, -2].mean() / 0.04 - 1.0) < 0.01
