"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).  TEST INFRASTRUCTURE ONLY.

The oracle restates the reference's solver hooks (lbm_oracle.cpp) and voxelizer
(voxel_oracle.cpp); see those files for the reference citations.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build
from lb_gb300.capi import LbmConfig, LbmBcInlet, LbmBcOutlet, LbmBcSymmetry, LbmDiag  # plain ctypes structs

_lib = None
# LBM_ORACLE_NATIVE=1 (set before the first call) loads the host-tuned build; bench.py's timed CPU
# baseline uses it, the parity tests keep the portable one
NATIVE = os.environ.get("LBM_ORACLE_NATIVE") == "1"


def lib():
    global _lib
    if _lib is None:
        path = _build.build(native=NATIVE)
        L = C.CDLL(path)
        vp, i32, f64 = C.c_void_p, C.c_int, C.c_double
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int32)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.POINTER(LbmConfig), i32, i32]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_threads.argtypes = [i32]
        L.orc_max_threads.restype = i32
        L.orc_host_stream_gbs.restype = f64
        L.orc_host_stream_gbs.argtypes = [C.c_longlong, i32]
        L.orc_set_flags.argtypes = [vp, ip]
        L.orc_set_bc.argtypes = [vp, C.POINTER(LbmBcInlet), i32, C.POINTER(LbmBcOutlet), i32]
        L.orc_set_periodic_list.argtypes = [vp, ip, i32]
        L.orc_set_symmetry.argtypes = [vp, C.POINTER(LbmBcSymmetry), i32]
        L.orc_set_wall_policy.argtypes = [vp, i32]
        L.orc_init_equilibrium.argtypes = [vp, f64, dp]
        L.orc_init_fields.argtypes = [vp, dp, dp]
        L.orc_step.argtypes = [vp, i32]
        L.orc_get_moments.argtypes = [vp, dp, dp]
        L.orc_get_omega.argtypes = [vp, dp]
        L.orc_get_df.argtypes = [vp, dp]
        L.orc_set_omega_next.argtypes = [vp, dp]
        L.orc_set_df.argtypes = [vp, dp]
        L.orc_timeavg_begin.argtypes = [vp]
        L.orc_timeavg_end.argtypes = [vp]
        L.orc_timeavg_get.argtypes = [vp, dp, dp, dp, C.POINTER(C.c_int64)]
        L.orc_error.argtypes = [vp, dp]
        L.orc_diag.argtypes = [vp, C.POINTER(LbmDiag)]
        L.orc_wall_list_size.argtypes = [vp]
        L.orc_wall_list_size.restype = i32
        L.orc_mesher_wall_pass.argtypes = [ip, i32, i32, i32]
        L.orc_collide_cell.argtypes = [i32, i32, dp, f64, dp, f64, dp, dp, i32, i32]
        L.orc_voxelize_off.argtypes = [C.c_char_p, f64, f64, dp, ip, ip, dp]
        L.orc_voxelize_mesh.argtypes = [dp, i32, ip, i32, f64, f64, dp, ip, ip, dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class OracleSim:
    """Reference-structured A-B solver (one omega, collision, streaming, boundary and moment
    pass per step).  precision 64 or 32."""

    def __init__(self, cfg, precision=64, ref_compat=False):
        self.cfg = cfg
        self.N = cfg.nx * cfg.ny * cfg.nz
        self.h = lib().orc_create(C.byref(cfg), precision, 1 if ref_compat else 0)
        if not self.h:
            raise ValueError("oracle: bad config")

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_flags(self, flags):
        f = np.ascontiguousarray(flags, dtype=np.int32).reshape(-1)
        assert f.size == self.N
        lib().orc_set_flags(self.h, _i(f))

    def set_bc(self, inlets=(), outlets=()):
        ni, no = len(inlets), len(outlets)
        ai = (LbmBcInlet * max(ni, 1))(*inlets)
        ao = (LbmBcOutlet * max(no, 1))(*outlets)
        lib().orc_set_bc(self.h, ai, ni, ao, no)

    def set_wall_policy(self, mesh_variant):
        """1: BounceBackWallHalfMesh (flag-2 cells under ref_compat), 0: BounceBackWallHalf (the list)."""
        lib().orc_set_wall_policy(self.h, int(mesh_variant))

    def set_symmetry(self, records=()):
        n = len(records)
        a = (LbmBcSymmetry * max(n, 1))(*records)
        lib().orc_set_symmetry(self.h, a, n)

    def set_periodic_list(self, recs):
        r = np.ascontiguousarray(recs, dtype=np.int32).reshape(-1, 8)
        lib().orc_set_periodic_list(self.h, _i(r), r.shape[0])

    def init_equilibrium(self, rho0=1.0, u0=(0.0, 0.0, 0.0)):
        u = np.asarray(u0, dtype=np.float64)
        lib().orc_init_equilibrium(self.h, float(rho0), _d(u))

    def init_fields(self, rho, u):
        r = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1)
        uu = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        lib().orc_init_fields(self.h, _d(r), _d(uu))

    def step(self, n=1):
        lib().orc_step(self.h, int(n))

    def moments(self):
        rho = np.empty(self.N)
        u = np.empty(3 * self.N)
        lib().orc_get_moments(self.h, _d(rho), _d(u))
        return rho, u.reshape(3, self.N)

    def omega(self):
        o = np.empty(self.N)
        lib().orc_get_omega(self.h, _d(o))
        return o

    def set_omega_next(self, omega):
        """Per-cell relaxation rate for the next step in place of the closure pass (one step)."""
        a = np.ascontiguousarray(omega, dtype=np.float64).reshape(-1)
        lib().orc_set_omega_next(self.h, _d(a))

    def populations(self):
        f = np.empty(27 * self.N)
        lib().orc_get_df(self.h, _d(f))
        return f.reshape(27, self.N)

    def set_populations(self, f):
        a = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        lib().orc_set_df(self.h, _d(a))

    def timeavg_begin(self):
        lib().orc_timeavg_begin(self.h)

    def timeavg_end(self):
        lib().orc_timeavg_end(self.h)

    def timeavg_get(self):
        r = np.empty(self.N)
        u = np.empty(3 * self.N)
        uu = np.empty(6 * self.N)
        cnt = C.c_int64(0)
        lib().orc_timeavg_get(self.h, _d(r), _d(u), _d(uu), C.byref(cnt))
        return r, u.reshape(3, self.N), uu.reshape(6, self.N), cnt.value

    def error(self):
        e = C.c_double(0)
        lib().orc_error(self.h, C.byref(e))
        return e.value

    def diag(self):
        d = LbmDiag()
        lib().orc_diag(self.h, C.byref(d))
        return d

    def wall_list_size(self):
        return lib().orc_wall_list_size(self.h)


def set_threads(n):
    lib().orc_set_threads(int(n))


def max_threads():
    return lib().orc_max_threads()


def host_stream_gbs(n=1 << 25, reps=4):
    """STREAM-triad bandwidth of the host's memory on all oracle threads (GB/s)."""
    return lib().orc_host_stream_gbs(int(n), int(reps))


def wall_pass(flags):
    f = np.ascontiguousarray(flags, dtype=np.int32)
    nz, ny, nx = f.shape
    lib().orc_mesher_wall_pass(_i(f), nx, ny, nz)
    return f


def collide_cell(f_in, rho, u, omega, collision, precision=64, force=(0.0, 0.0, 0.0), ref_compat=False, flag=1):
    """One collision of a single cell whose reference flag is `flag` (the combined collision picks its
    operator by flag: 1 -> cumulant-2015, other -> cumulant-2017)."""
    fi = np.ascontiguousarray(f_in, dtype=np.float64)
    uu = np.ascontiguousarray(u, dtype=np.float64)
    ff = np.ascontiguousarray(force, dtype=np.float64)
    out = np.empty(27)
    lib().orc_collide_cell(precision, collision, _d(fi), float(rho), _d(uu), float(omega), _d(ff), _d(out),
                           int(ref_compat), int(flag))
    return out


def voxelize_off(path, res, add, outside=(-1.0, -1.0, -1.0)):
    """Reference voxelizer restated: returns (flags[z,y,x] int32, bbox(6))."""
    o = np.asarray(outside, dtype=np.float64)
    dims = np.zeros(3, dtype=np.int32)
    bbox = np.zeros(6)
    rc = lib().orc_voxelize_off(path.encode(), float(res), float(add), _d(o), None, _i(dims), _d(bbox))
    if rc != 0:
        raise IOError(f"oracle could not read {path}")
    flags = np.zeros(int(dims.prod()), dtype=np.int32)
    lib().orc_voxelize_off(path.encode(), float(res), float(add), _d(o), _i(flags), _i(dims), _d(bbox))
    return flags.reshape(dims[2], dims[1], dims[0]), bbox


def voxelize_mesh(verts, tris, res, add, outside):
    v = np.ascontiguousarray(verts, dtype=np.float64)
    t = np.ascontiguousarray(tris, dtype=np.int32)
    o = np.asarray(outside, dtype=np.float64)
    dims = np.zeros(3, dtype=np.int32)
    bbox = np.zeros(6)
    lib().orc_voxelize_mesh(_d(v), v.shape[0], _i(t), t.shape[0], float(res), float(add), _d(o), None, _i(dims), _d(bbox))
    flags = np.zeros(int(dims.prod()), dtype=np.int32)
    lib().orc_voxelize_mesh(_d(v), v.shape[0], _i(t), t.shape[0], float(res), float(add), _d(o), _i(flags), _i(dims), _d(bbox))
    return flags.reshape(dims[2], dims[1], dims[0]), bbox
