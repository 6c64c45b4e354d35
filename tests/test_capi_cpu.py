"""The C-ABI library builds, loads without a GPU and exports every function include/lbm.h declares."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from lb_gb300 import capi

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "lbm.h")


def declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(lbm_\w+)\s*\(", txt)))


def test_header_declares_entry_points():
    names = declared()
    assert "lbm_create" in names and "lbm_step" in names and "lbm_voxelize_off" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(built_lib):
    L = C.CDLL(built_lib)
    missing = [n for n in declared() if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings_and_abi(built_lib):
    L = capi.lib()
    assert L.lbm_abi_version() == 3
    assert L.lbm_status_string(capi.LBM_ERR_NONFINITE) == b"non-finite populations"


def test_create_rejects_bad_config_before_touching_the_gpu(built_lib):
    L = capi.lib()
    ctx = C.c_void_p()
    cfg = capi.make_config(2, 8, 8)
    assert L.lbm_create(C.byref(cfg), C.byref(ctx)) == capi.LBM_ERR_INVALID
    cfg = capi.make_config(8, 8, 8, nu=-0.2)
    assert L.lbm_create(C.byref(cfg), C.byref(ctx)) == capi.LBM_ERR_INVALID
    cfg = capi.make_config(8, 8, 8, closure=7)
    assert L.lbm_create(C.byref(cfg), C.byref(ctx)) == capi.LBM_ERR_UNSUPPORTED
    cfg = capi.make_config(2048, 1024, 1024)  # 2^31 cells: beyond the 32-bit cell index
    assert L.lbm_create(C.byref(cfg), C.byref(ctx)) == capi.LBM_ERR_UNSUPPORTED
    cfg = capi.make_config(8, 70000, 8)  # beyond the launch grid's y extent
    assert L.lbm_create(C.byref(cfg), C.byref(ctx)) == capi.LBM_ERR_UNSUPPORTED
    cfg = capi.make_config(8, 8, 8, collision=5)
    assert L.lbm_create(C.byref(cfg), C.byref(ctx)) == capi.LBM_ERR_UNSUPPORTED
    cfg = capi.make_config(8, 8, 8, collision=capi.LBM_COLLISION_CUMULANT2017, closure=capi.LBM_CLOSURE_MLP,
                           storage=capi.LBM_STORAGE_F32)  # the learned closure: SRT or cumulant-2015
    assert L.lbm_create(C.byref(cfg), C.byref(ctx)) == capi.LBM_ERR_UNSUPPORTED
    cfg = capi.make_config(8, 8, 8, inlet_kind=3)
    assert L.lbm_create(C.byref(cfg), C.byref(ctx)) == capi.LBM_ERR_UNSUPPORTED
    cfg = capi.make_config(8, 8, 8, outlet_kind=5)
    assert L.lbm_create(C.byref(cfg), C.byref(ctx)) == capi.LBM_ERR_UNSUPPORTED
    cfg = capi.make_config(8, 8, 8, closure=capi.LBM_CLOSURE_MLP, storage=capi.LBM_STORAGE_F16DEV,
                           outlet_kind=capi.LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA)  # sponge + learned closure
    assert L.lbm_create(C.byref(cfg), C.byref(ctx)) == capi.LBM_ERR_UNSUPPORTED


def test_mesher_wall_pass_host_only(built_lib):
    f = np.ones((4, 5, 6), np.int32)
    f[:, 0, :] = 0
    ptr = f.ctypes.data_as(C.POINTER(C.c_int32))
    assert capi.lib().lbm_mesher_wall_pass(ptr, 6, 5, 4) == 0
    assert f[1, 1, 2] == 1 + 9 and f[1, 2, 2] == 1 and f[0, 1, 2] == 1 + 6


def test_laminar_collisions_run_with_the_global_omega():
    """CollisionSRTLaminar, CollisionSRTunroll and CollisionCumD3Q27Laminar read Constants->omega
    (CollisionSRTLaminar.h:28, CollisionSRTunroll.h:27, CollisionCumD3Q27Laminar.h:27), never the
    per-cell field that OmegaLES and the outlet sponge write: the mirror gives them no closure and a
    sponge of slope 0, and keeps the turbulent collisions' choices."""
    from lb_gb300 import solver as S
    for coll, code in ((S.CollisionSRTLaminar, capi.LBM_COLLISION_SRT), (S.CollisionSRTunroll, capi.LBM_COLLISION_SRT),
                       (S.CollisionCumD3Q27Laminar, capi.LBM_COLLISION_CUMULANT2015)):
        assert coll.code == code
        for turb in (S.OmegaLES, S.OmegaMLP, S.OmegaNo):
            t, d = S.effective_closure(coll, turb, (0.0, 0.05))
            assert t is S.OmegaNo and d == (0.0, 0.0)
    for coll in (S.CollisionSRTTurbulent, S.CollisionCumD3Q27Turbulent2015, S.CollisionCumD3Q27Turbulent2017,
                 S.CollisionCumD3Q27TurbulentCombined):
        assert S.effective_closure(coll, S.OmegaLES, (0.0, 0.05)) == (S.OmegaLES, (0.0, 0.05))


def test_case_file_fills_the_config(built_lib):
    """lbm_config_parse: a case file with the reference's policy names and the field names of lbm_config
    gives the config make_config builds from the same values; unknown keys and bad values are refused
    with the line named and the config left as it was."""
    text = """
    # turbulent duct, as main.cu sets one up
    nx = 96
    ny 48
    nz=48
    periodic 0 1 1
    collision = CollisionCumD3Q27Turbulent2017
    closure = OmegaLES          # Smagorinsky
    storage f16dev
    inlet = InletVelocityZouHe
    outlet = OutletNeighbourEquilibriumOmegaRF
    nu = 0.002
    cles 0.17
    force 1e-7, 0, 0
    omega_dumping 0.0 0.05
    mlp_interval 16
    """
    c = capi.config_from_text(text)
    want = capi.make_config(96, 48, 48, periodic=(0, 1, 1), collision=capi.LBM_COLLISION_CUMULANT2017,
                            closure=capi.LBM_CLOSURE_SMAGORINSKY, storage=capi.LBM_STORAGE_F16DEV,
                            inlet_kind=capi.LBM_INLET_ZOU_HE, nu=0.002, cles=0.17, force=(1e-7, 0, 0),
                            outlet_kind=capi.LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA_RF, omega_dumping=(0.0, 0.05),
                            mlp_interval=16)
    assert bytes(c) == bytes(want)
    d = capi.config_from_text("")
    assert bytes(d) == bytes(capi.make_config(0, 0, 0))
    assert capi.config_from_text("collision srt\nstorage 0", base=c).collision == capi.LBM_COLLISION_SRT
    from lb_gb300.solver import Solver
    with pytest.raises(capi.LbmError) as e:  # refused by the set-up checks, before any device work
        Solver.from_config(capi.config_from_text("nx 8\nny 8\nnz 8\ncollision 5"))
    assert e.value.status == capi.LBM_ERR_UNSUPPORTED
    for bad in ("nx = 9x", "periodic 1 1", "colision srt", "closure smagorinski", "tau"):
        with pytest.raises(capi.LbmError) as e:
            capi.config_from_text("nx 8\n" + bad, base=c)
        assert e.value.status == capi.LBM_ERR_INVALID and "line 2" in str(e.value)
