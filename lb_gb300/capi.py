"""ctypes mirror of include/lbm.h and the loader of the in-tree CUDA library.

The shared library lb_gb300/liblbm_gb300.so is built by lb_gb300.build (nvcc, sm_103a).
Loading fails loudly when it is missing: there is no CPU fallback in the product path.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblbm_gb300.so")

LBM_OK = 0
LBM_ERR_INVALID = -1
LBM_ERR_OOM = -2
LBM_ERR_CUDA = -3
LBM_ERR_NONFINITE = -4
LBM_ERR_TIMEOUT = -5
LBM_ERR_STATE = -6
LBM_ERR_IO = -7
LBM_ERR_UNSUPPORTED = -8

LBM_COLLISION_SRT = 0
LBM_COLLISION_CUMULANT2015 = 1
LBM_COLLISION_CUMULANT2017 = 2
LBM_COLLISION_CUMULANT_COMBINED = 3
LBM_CLOSURE_NONE = 0
LBM_CLOSURE_SMAGORINSKY = 1
LBM_CLOSURE_MLP = 2
LBM_STORAGE_F64 = 0
LBM_STORAGE_F32 = 1
LBM_STORAGE_F16DEV = 2
LBM_INLET_MOVING_WALL = 0
LBM_INLET_EQUILIBRIUM = 1
LBM_INLET_ZOU_HE = 2
LBM_OUTLET_DENSITY_INTERPOLATED = 0
LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM = 1
LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA = 2
LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA_RF = 3
LBM_OUTLET_DENSITY_EQUILIBRIUM = 4


class LbmConfig(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("periodic", C.c_int32 * 3),
        ("collision", C.c_int32), ("closure", C.c_int32), ("storage", C.c_int32),
        ("inlet_kind", C.c_int32),
        ("nu", C.c_double), ("tau", C.c_double), ("cles", C.c_double),
        ("force", C.c_double * 3),
        ("rho0", C.c_double),
        ("f16_scale_log2", C.c_int32),
        ("device", C.c_int32),
        ("options", C.c_int32),
        ("mlp_interval", C.c_int32),
        ("outlet_kind", C.c_int32),
        ("omega_dumping_low", C.c_double), ("omega_dumping_high", C.c_double),
    ]


LBM_OPT_ROW_STAGING = 1
LBM_OPT_F16_ROUND_NEAREST = 2
LBM_OPT_ONE_LAUNCH = 4
LBM_OPT_NO_WALL_ROWS = 8
LBM_OPT_MLP_TCGEN05 = 16
LBM_MLP_PATH_WARP_MMA, LBM_MLP_PATH_TCGEN05 = 0, 1


LBM_MLP_INPUTS = 7
LBM_MLP_HIDDEN = 32
LBM_MLP_PARAMS = LBM_MLP_HIDDEN * LBM_MLP_HIDDEN + 10 * LBM_MLP_HIDDEN + 1
LBM_MLP_SAMPLE = 10


class LbmMlpModel(C.Structure):
    _fields_ = [("params", C.c_float * LBM_MLP_PARAMS),
                ("in_mean", C.c_float * LBM_MLP_INPUTS), ("in_std", C.c_float * LBM_MLP_INPUTS),
                ("in_lo", C.c_float * LBM_MLP_INPUTS), ("in_hi", C.c_float * LBM_MLP_INPUTS),
                ("out_scale", C.c_float)]


class LbmVertex(C.Structure):
    _fields_ = [("x", C.c_int32), ("y", C.c_int32), ("z", C.c_int32)]


class LbmBcInlet(C.Structure):
    _fields_ = [("vertex", LbmVertex), ("normal", C.c_float * 3), ("velocity", C.c_float * 3),
                ("regular", C.c_int32)]


class LbmBcOutlet(C.Structure):
    _fields_ = [("vertex", LbmVertex), ("normal", C.c_float * 3), ("density", C.c_float),
                ("regular", C.c_int32)]


class LbmBcSymmetry(C.Structure):
    _fields_ = [("vertex", LbmVertex), ("normal", C.c_float * 3), ("regular", C.c_int32)]


class LbmBcPeriodic(C.Structure):
    _fields_ = [("vertex", LbmVertex), ("normal", C.c_float * 3), ("periodic_index", C.c_int32),
                ("regular", C.c_int32)]


class LbmMeshFrame(C.Structure):
    _fields_ = [("dims", C.c_int32 * 3), ("resolution_factor", C.c_float), ("additional_factor", C.c_float),
                ("bbmin", C.c_float * 3)]


class LbmCuboid(C.Structure):
    _fields_ = [("x1", C.c_double * 3), ("x2", C.c_double * 3), ("x3", C.c_double * 3), ("id", C.c_int32)]


class LbmVtkField(C.Structure):
    _fields_ = [("name", C.c_char_p), ("components", C.c_int32), ("data", C.POINTER(C.c_double)),
                ("scale", C.c_double)]


class LbmDiag(C.Structure):
    _fields_ = [("mass", C.c_double), ("momentum", C.c_double * 3), ("drag", C.c_double * 3),
                ("max_speed", C.c_double), ("nonfinite", C.c_int64), ("fluid_cells", C.c_int64),
                ("step", C.c_int64)]


def make_config(nx, ny, nz, periodic=(0, 0, 0), collision=LBM_COLLISION_CUMULANT2015,
                closure=LBM_CLOSURE_NONE, storage=LBM_STORAGE_F32, inlet_kind=LBM_INLET_MOVING_WALL,
                nu=1.0 / 6.0, tau=0.0, cles=0.173, force=(0.0, 0.0, 0.0), rho0=1.0,
                f16_scale_log2=10, device=0, options=0, mlp_interval=1, outlet_kind=LBM_OUTLET_DENSITY_INTERPOLATED,
                omega_dumping=(-1.0, -1.0)):
    c = LbmConfig()
    c.nx, c.ny, c.nz = int(nx), int(ny), int(nz)
    for a in range(3):
        c.periodic[a] = int(periodic[a])
        c.force[a] = float(force[a])
    c.collision, c.closure, c.storage, c.inlet_kind = int(collision), int(closure), int(storage), int(inlet_kind)
    c.nu, c.tau, c.cles, c.rho0 = float(nu), float(tau), float(cles), float(rho0)
    c.f16_scale_log2, c.device, c.options = int(f16_scale_log2), int(device), int(options)
    c.mlp_interval = int(mlp_interval)
    c.outlet_kind = int(outlet_kind)
    c.omega_dumping_low, c.omega_dumping_high = float(omega_dumping[0]), float(omega_dumping[1])
    return c


def config_from_text(text, base=None):
    """lbm_config_parse: a key = value case file over `base` (default: lbm_config_defaults)."""
    c = LbmConfig()
    if base is None:
        lib().lbm_config_defaults(C.byref(c))
    else:
        C.memmove(C.byref(c), C.byref(base), C.sizeof(LbmConfig))
    st = lib().lbm_config_parse(text.encode(), C.byref(c))
    if st:
        raise LbmError(st, lib().lbm_config_last_error().decode())
    return c


def make_inlet(x, y, z, normal, velocity, regular=1):
    r = LbmBcInlet()
    r.vertex = LbmVertex(int(x), int(y), int(z))
    for a in range(3):
        r.normal[a] = float(normal[a])
        r.velocity[a] = float(velocity[a])
    r.regular = int(regular)
    return r


def make_outlet(x, y, z, normal, density, regular=1):
    r = LbmBcOutlet()
    r.vertex = LbmVertex(int(x), int(y), int(z))
    for a in range(3):
        r.normal[a] = float(normal[a])
    r.density = float(density)
    r.regular = int(regular)
    return r


def make_symmetry(x, y, z, normal, regular=1):
    r = LbmBcSymmetry()
    r.vertex = LbmVertex(int(x), int(y), int(z))
    for a in range(3):
        r.normal[a] = float(normal[a])
    r.regular = int(regular)
    return r


class LbmError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"lbm status {status}: {msg}")
        self.status = status


_lib = None


def lib():
    """Load liblbm_gb300.so; raises if the CUDA library has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with lb_gb300.build.build() "
                          "(the solver has no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    vp, i32, f64 = C.c_void_p, C.c_int32, C.c_double
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
    fp, i64 = C.POINTER(C.c_float), C.c_int64
    sig = {
        "lbm_create": ([C.POINTER(LbmConfig), C.POINTER(vp)], i32),
        "lbm_destroy": ([vp], i32),
        "lbm_status_string": ([i32], C.c_char_p),
        "lbm_last_error": ([vp], C.c_char_p),
        "lbm_abi_version": ([], i32),
        "lbm_set_flags": ([vp, ip], i32),
        "lbm_set_bc": ([vp, C.POINTER(LbmBcInlet), i32, C.POINTER(LbmBcOutlet), i32], i32),
        "lbm_set_symmetry": ([vp, C.POINTER(LbmBcSymmetry), i32], i32),
        "lbm_init_equilibrium": ([vp, f64, dp], i32),
        "lbm_init_fields": ([vp, dp, dp], i32),
        "lbm_step": ([vp, i32], i32),
        "lbm_synchronize": ([vp], i32),
        "lbm_step_timed": ([vp, i32, dp], i32),
        "lbm_step_launches": ([vp, ip], i32),
        "lbm_get_eddy_viscosity": ([vp, dp], i32),
        "lbm_probe": ([vp, i32, i32, i32, dp], i32),
        "lbm_get_moments": ([vp, dp, dp], i32),
        "lbm_get_populations": ([vp, dp], i32),
        "lbm_set_populations": ([vp, dp], i32),
        "lbm_reduce": ([vp, C.POINTER(LbmDiag)], i32),
        "lbm_error_evaluation": ([vp, dp], i32),
        "lbm_timeavg_begin": ([vp], i32),
        "lbm_timeavg_end": ([vp], i32),
        "lbm_timeavg_get": ([vp, dp, dp, dp, C.POINTER(C.c_int64)], i32),
        "lbm_checkpoint_save": ([vp, C.c_char_p], i32),
        "lbm_checkpoint_load": ([vp, C.c_char_p], i32),
        "lbm_mesher_wall_pass": ([ip, i32, i32, i32], i32),
        "lbm_voxelize_off": ([C.c_char_p, f64, f64, dp, ip, ip, dp, i32], i32),
        "lbm_voxelize_mesh": ([dp, i32, ip, i32, f64, f64, ip, ip, dp, i32], i32),
        "lbm_voxelize_mesh_noalloc": ([dp, i32, ip, i32, f64, f64, C.c_void_p, ip, dp, i32], i32),
        "lbm_mlp_load": ([vp, C.POINTER(LbmMlpModel)], i32),
        "lbm_les_samples": ([vp, i32, fp, i64, C.POINTER(i64)], i32),
        "lbm_mlp_eval": ([C.POINTER(LbmMlpModel), fp, i64, fp, ip, i32], i32),
        "lbm_mlp_eval_path": ([C.POINTER(LbmMlpModel), fp, i64, fp, ip, i32, i32], i32),
        "lbm_mlp_trainer_create": ([fp, i64, i32, C.POINTER(vp)], i32),
        "lbm_mlp_trainer_destroy": ([vp], i32),
        "lbm_mlp_trainer_norm": ([vp], f64),
        "lbm_mlp_gradient": ([vp, C.POINTER(LbmMlpModel), i64, i64, fp, dp], i32),
        "lbm_mlp_train": ([vp, C.POINTER(LbmMlpModel), i32, i32, C.c_float, C.c_uint64, fp], i32),
        "lbm_mlp_last_error": ([], C.c_char_p),
        "lbm_mesh_matrix_write": ([C.c_char_p, ip, ip, f64, f64, dp], i32),
        "lbm_mesh_matrix_read": ([C.c_char_p, ip, i64, ip, dp, dp, dp], i32),
        "lbm_mesh_matrix_last_error": ([], C.c_char_p),
        "lbm_vtk_write": ([C.c_char_p, C.c_char_p, ip, f64, f64, dp, C.POINTER(LbmVtkField), i32], i32),
        "lbm_probe_csv_append": ([C.c_char_p, f64, dp, f64, f64, f64], i32),
        "lbm_vtk_read_variables": ([C.c_char_p, ip, dp, dp], i32),
        "lbm_mesher_inlet_uniform": ([C.POINTER(LbmMeshFrame), ip, C.POINTER(LbmCuboid), fp, fp,
                                      C.POINTER(LbmBcInlet), i64, C.POINTER(C.c_int64)], i32),
        "lbm_mesher_inlet_paraboloid_circle": ([C.POINTER(LbmMeshFrame), ip, C.POINTER(LbmCuboid), dp, C.c_float, fp,
                                                C.c_float, C.POINTER(LbmBcInlet), i64, C.POINTER(C.c_int64)], i32),
        "lbm_mesher_inlet_paraboloid_rectangle": ([C.POINTER(LbmMeshFrame), ip, C.POINTER(LbmCuboid), dp, fp, fp,
                                                   C.c_float, C.POINTER(LbmBcInlet), i64, C.POINTER(C.c_int64)], i32),
        "lbm_mesher_outlet": ([C.POINTER(LbmMeshFrame), ip, C.POINTER(LbmCuboid), fp, C.c_float,
                               C.POINTER(LbmBcOutlet), i64, C.POINTER(C.c_int64)], i32),
        "lbm_mesher_symmetry": ([C.POINTER(LbmMeshFrame), ip, C.POINTER(LbmCuboid), fp, C.POINTER(LbmBcSymmetry), i64,
                                 C.POINTER(C.c_int64)], i32),
        "lbm_mesher_periodic": ([C.POINTER(LbmMeshFrame), ip, C.POINTER(LbmCuboid), fp, i32, C.POINTER(LbmBcPeriodic),
                                 i64, C.POINTER(C.c_int64)], i32),
        "lbm_mesher_last_error": ([], C.c_char_p),
        "lbm_config_defaults": ([C.POINTER(LbmConfig)], i32),
        "lbm_config_parse": ([C.c_char_p, C.POINTER(LbmConfig)], i32),
        "lbm_config_last_error": ([], C.c_char_p),
        "lbm_vtk_last_error": ([], C.c_char_p),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def check(status, ctx=None, mlp=False):
    if status != LBM_OK:
        L = lib()
        msg = L.lbm_mlp_last_error() if mlp else L.lbm_last_error(ctx)
        raise LbmError(status, (msg or b"").decode() or L.lbm_status_string(status).decode())
    return status
