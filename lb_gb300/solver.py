"""Host-side mirror of the reference's solver/plugin interface over the C ABI (include/lbm.h).

The reference composes a solver from compile-time policy structs
(3D/simulation/src/solvers/SolverTurbulentLES.h:67-82, chosen in 3D/simulation/main.cu:37-52):

    SolverTurbulentLES<Model, Initialisation, Collision, Streaming, BounceBackWall, Symmetry,
                       Periodic, Inlet, Outlet, Moments, Turbulence, Error, NonDim, TimeAvg>

Here the same policy names are tags that select the fused kernel's operator.  `Solver` is the
thin object over one lbm_ctx; `SolverTurbulentLES` keeps the reference's method names
(convertToLattice, initializeSimulation, runSimulation).  Every call goes to the CUDA library;
there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

from . import capi
from .capi import check, lib


# ---- policy tags (reference names) ---------------------------------------------------------------
class D3Q27:                                    # models/D3Q27/D3Q27.h
    numberOfDiscreteVelocities = 27


class CollisionCumD3Q27Turbulent2015:           # collisions/CollisionCumD3Q27Turbulent2015.h
    code = capi.LBM_COLLISION_CUMULANT2015


class CollisionCumD3Q27Turbulent2017:           # collisions/CollisionCumD3Q27Turbulent2017.h
    code = capi.LBM_COLLISION_CUMULANT2017


class CollisionCumD3Q27TurbulentCombined:       # collisions/CollisionCumD3Q27TurbulentCombined.h
    code = capi.LBM_COLLISION_CUMULANT_COMBINED


class CollisionSRTTurbulent:                    # collisions/CollisionSRTTurbulent.h
    code = capi.LBM_COLLISION_SRT


class CollisionSRTLaminar(CollisionSRTTurbulent):
    """collisions/CollisionSRTLaminar.h: the SRT update with the global omega = 1/tau (Constants->omega,
    :28); the solver then runs no closure and no outlet sponge, which the reference's laminar collisions
    ignore as they never read the per-cell field."""
    laminar = True


class CollisionSRTunroll(CollisionSRTLaminar):  # collisions/CollisionSRTunroll.h: CollisionSRTLaminar unrolled
    pass


class CollisionCumD3Q27Laminar(CollisionCumD3Q27Turbulent2015):
    """collisions/CollisionCumD3Q27Laminar.h: the 2015 cumulant with omega1 = the global 1/tau (:27)."""
    laminar = True


class OmegaLES:                                 # turbulence/OmegaLES.h
    code = capi.LBM_CLOSURE_SMAGORINSKY


class OmegaNo:                                  # turbulence/OmegaNo.h
    code = capi.LBM_CLOSURE_NONE


class OmegaMLP:                                 # learned closure (lb_gb300.les); no reference policy
    code = capi.LBM_CLOSURE_MLP


class StreamingAB:                              # streamings/StreamingAB.h (AA in place here)
    pass


class BounceBackWallHalf:                       # boundaryConditions/Wall/BounceBackWallHalf.h
    pass


class BounceBackWallHalfMesh(BounceBackWallHalf):  # boundaryConditions/Wall/BounceBackWallHalfMesh.h: the same
    pass                                           # rule on every fluid cell with a solid neighbour


class NoSymmetry:                               # boundaryConditions/Symmetry/NoSymmetry.h
    pass


class BounceSymmetryHalf:                       # boundaryConditions/Symmetry/BounceSymmetryHalf.h (+-y normals)
    pass


class Periodic:                                 # boundaryConditions/Periodic/Periodic.h (index wrap here)
    pass


class NoPeriodic:
    pass


class InletVelocityMovingWall:                  # boundaryConditions/Inlet/InletVelocityMovingWall.h
    code = capi.LBM_INLET_MOVING_WALL


class InletVelocityEquilibrium:                 # boundaryConditions/Inlet/InletVelocityEquilibrium.h
    code = capi.LBM_INLET_EQUILIBRIUM


class InletVelocityZouHe:                       # boundaryConditions/Inlet/InletVelocityZouHe.h
    code = capi.LBM_INLET_ZOU_HE


class OutletDensityInterpolated:                # boundaryConditions/Outlet/OutletDensityInterpolated.h
    code = capi.LBM_OUTLET_DENSITY_INTERPOLATED


class OutletNeighbourEquilibrium:               # boundaryConditions/Outlet/OutletNeighbourEquilibrium.h
    code = capi.LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM


class OutletNeighbourEquilibriumOmega:          # .../Outlet/OutletNeighbourEquilibriumOmega.h (+ sponge)
    code = capi.LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA


class OutletNeighbourEquilibriumOmegaRF:        # .../Outlet/OutletNeighbourEquilibriumOmegaRF.h
    code = capi.LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA_RF


class OutletDensityEquilibrium:                 # boundaryConditions/Outlet/OutletDensityEquilibrium.h
    code = capi.LBM_OUTLET_DENSITY_EQUILIBRIUM


class MomentDensityVelocityN27:                 # moments/MomentDensityVelocityN27.h
    pass


class ErrorQuadratic:                           # errorEvaluations/ErrorQuadratic.h
    pass


class MomentTimeAvg:                            # moments/MomentTimeAvg.h
    pass


class InitializationEquilibriumConstVector:     # initializations/InitializationEquilibriumConstVector.h
    pass


class InitializationEquilibriumVariables:       # initializations/InitializationEquilibriumVariables.h
    """Restart: rho and u from the VTK file <results_dir>/<InitFileName> (a variablesLatticeVTK dump),
    inlet nodes at their record velocity, populations at equilibrium."""


class NonDimensiolnaliseFactorsVelocity:        # nonDimensionalisions/NonDimensiolnaliseFactorsVelocity.h
    """Physical -> lattice conversion (:20-131).  tau = 3 nu_lb + 1/2 here; the reference writes
    nu_lb/3 + 1/2 (:66), which `reference_tau` reproduces for comparison."""

    @staticmethod
    def factors(L_phys, nx, u_phys, U_lb, nu_phys, rho_phys):
        Cl = L_phys / nx
        Cu = u_phys / U_lb
        Ct = Cl / Cu
        nu_lb = nu_phys * Ct / Cl / Cl
        return {"Cl": Cl, "Cu": Cu, "Ct": Ct, "Cm": rho_phys * Cl ** 3, "nu": nu_lb, "tau": 3.0 * nu_lb + 0.5,
                "Re": u_phys * L_phys / nu_phys}

    @staticmethod
    def reference_tau(nu_lb):
        return nu_lb / 3.0 + 0.5

    @staticmethod
    def nonDimensionalize(c, nx):
        """nonDimensionalize (:20-85) on a constants dict, in the reference's float arithmetic: reads BBmin,
        BBmax, conversion_factor_fyz, u_guess_fyz, U_lb, rho_fyz, ny_fyz; sets L_fyz, Cl, Cu, Cu_inverse, Ct,
        Crho, Cm, Cpressure, Re, nu, tau, omega.  tau = 3 nu + 1/2 (nu / 3 + 1/2 with tau_ref_compat).
        U_lb >= cs or tau outside (0.5, 0.99) raise, where the reference asserts (:29, :81)."""
        f = np.float32
        with np.errstate(all="ignore"):
            if not f(c["U_lb"]) < f(1.0) / np.sqrt(f(3.0)):
                raise ValueError("U_lb must be below the speed of sound")
            L = f(abs(f(c["BBmax"][0]) - f(c["BBmin"][0]))) * f(c.get("conversion_factor_fyz", 1.0))
            Cl = L / f(nx)
            Cu = f(c["u_guess_fyz"]) / f(c["U_lb"])
            Ct = Cl / Cu
            Crho = f(c.get("rho_fyz", 1.0))
            Cm = Crho * Cl * Cl * Cl
            ny = f(c["ny_fyz"]) * Ct / Cl / Cl
            tau = ny / f(3.0) + f(0.5) if c.get("tau_ref_compat") else f(3.0) * ny + f(0.5)
        if not (f(0.5) < tau < f(0.99)):
            raise ValueError(f"tau = {float(tau)} outside (0.5, 0.99): change the resolution or the lattice speed")
        c.update(L_fyz=float(L), Cl=float(Cl), Cu=float(Cu), Cu_inverse=float(f(1.0) / Cu), Ct=float(Ct),
                 Crho=float(Crho), Cm=float(Cm), Cpressure=float(Cm / Cl / Ct / Ct),
                 Re=float(f(c["u_guess_fyz"]) * L / f(c["ny_fyz"])), nu=float(ny), tau=float(tau),
                 omega=float(f(1.0) / tau))
        return c

    @staticmethod
    def nonDimensionalizeInlet(records, c):
        """:87-108: inlet velocities times Cu_inverse (float); returns converted copies."""
        k = np.float32(c["Cu_inverse"])
        return [capi.make_inlet(r.vertex.x, r.vertex.y, r.vertex.z, tuple(r.normal),
                                [float(np.float32(v) * k) for v in r.velocity], r.regular) for r in records]

    @staticmethod
    def nonDimensionalizeOutlet(records, c):
        """:110-130: outlet densities / Cm * Cl^3 (float); returns converted copies."""
        Cm, Cl = np.float32(c["Cm"]), np.float32(c["Cl"])
        return [capi.make_outlet(r.vertex.x, r.vertex.y, r.vertex.z, tuple(r.normal),
                                 float(np.float32(r.density) / Cm * Cl * Cl * Cl), r.regular) for r in records]


STORAGE = {"f64": capi.LBM_STORAGE_F64, "f32": capi.LBM_STORAGE_F32, "f16dev": capi.LBM_STORAGE_F16DEV}


class Diag:
    def __init__(self, d):
        self.mass = d.mass
        self.momentum = tuple(d.momentum)
        self.drag = tuple(d.drag)
        self.max_speed = d.max_speed
        self.nonfinite = d.nonfinite
        self.fluid_cells = d.fluid_cells
        self.step = d.step


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def effective_closure(collision, turbulence, omega_dumping):
    """The closure and sponge a collision policy runs with: a laminar collision relaxes with the global
    1/tau whatever the turbulence and outlet policies compute, so it gets OmegaNo and a sponge of slope 0."""
    if getattr(collision, "laminar", False):
        return OmegaNo, (0.0, 0.0)
    return turbulence, omega_dumping


class Solver:
    """One lattice on one GPU (one lbm_ctx)."""

    def __init__(self, shape, collision=CollisionCumD3Q27Turbulent2015, turbulence=OmegaNo,
                 inlet=InletVelocityMovingWall, storage="f32", nu=1.0 / 6.0, tau=0.0, cles=0.173,
                 periodic=(0, 0, 0), force=(0.0, 0.0, 0.0), rho0=1.0, f16_scale_log2=10, device=0, options=0,
                 mlp_interval=1, outlet=OutletDensityInterpolated, omega_dumping=(-1.0, -1.0)):
        turbulence, omega_dumping = effective_closure(collision, turbulence, omega_dumping)
        nx, ny, nz = shape
        self.shape = (int(nx), int(ny), int(nz))
        self.N = nx * ny * nz
        self.cfg = capi.make_config(nx, ny, nz, periodic=periodic, collision=collision.code,
                                    closure=turbulence.code, storage=STORAGE[storage],
                                    inlet_kind=inlet.code, nu=nu, tau=tau, cles=cles, force=force,
                                    rho0=rho0, f16_scale_log2=f16_scale_log2, device=device, options=options,
                                    mlp_interval=mlp_interval, outlet_kind=outlet.code, omega_dumping=omega_dumping)
        self._ctx = C.c_void_p()
        check(lib().lbm_create(C.byref(self.cfg), C.byref(self._ctx)))

    @classmethod
    def from_config(cls, cfg):
        """A solver for a ready lbm_config, e.g. capi.config_from_text(case_file_text).  The config is used
        as given (no laminar-collision mapping: the case file names the closure itself)."""
        s = cls.__new__(cls)
        s.shape = (int(cfg.nx), int(cfg.ny), int(cfg.nz))
        s.N = s.shape[0] * s.shape[1] * s.shape[2]
        s.cfg = capi.LbmConfig()
        C.memmove(C.byref(s.cfg), C.byref(cfg), C.sizeof(capi.LbmConfig))
        s._ctx = C.c_void_p()
        check(lib().lbm_create(C.byref(s.cfg), C.byref(s._ctx)))
        return s

    # -- lifecycle
    def close(self):
        if self._ctx:
            lib().lbm_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, s):
        return check(s, self._ctx)

    # -- set-up
    def set_flags(self, flags):
        """flags: int32 array [z, y, x] in the reference encoding (0 solid, >0 fluid, -1, -2, -3)."""
        f = np.ascontiguousarray(flags, dtype=np.int32).reshape(-1)
        assert f.size == self.N
        self._check(lib().lbm_set_flags(self._ctx, f.ctypes.data_as(C.POINTER(C.c_int32))))

    def set_bc(self, inlets=(), outlets=()):
        ni, no = len(inlets), len(outlets)
        ai = (capi.LbmBcInlet * max(ni, 1))(*inlets)
        ao = (capi.LbmBcOutlet * max(no, 1))(*outlets)
        self._check(lib().lbm_set_bc(self._ctx, ai, ni, ao, no))

    def set_symmetry(self, records=()):
        """BounceSymmetryHalf records (capi.make_symmetry) of -2 nodes; call after set_bc."""
        n = len(records)
        a = (capi.LbmBcSymmetry * max(n, 1))(*records)
        self._check(lib().lbm_set_symmetry(self._ctx, a, n))

    def init_equilibrium(self, rho0=1.0, u0=(0.0, 0.0, 0.0)):
        u = np.asarray(u0, dtype=np.float64)
        self._check(lib().lbm_init_equilibrium(self._ctx, float(rho0), _dp(u)))

    def init_fields(self, rho, u):
        r = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1)
        uu = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        self._check(lib().lbm_init_fields(self._ctx, _dp(r), _dp(uu)))

    def set_populations(self, f):
        a = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        self._check(lib().lbm_set_populations(self._ctx, _dp(a)))

    # -- stepping
    def step(self, n=1):
        self._check(lib().lbm_step(self._ctx, int(n)))

    def step_timed(self, n):
        """n steps timed with CUDA events on the context's stream; returns milliseconds."""
        ms = C.c_double(0)
        self._check(lib().lbm_step_timed(self._ctx, int(n), C.byref(ms)))
        return ms.value

    def eddy_viscosity(self):
        """The learned closure's kept nu_t per cell (mlp_interval > 1): -1 where the cell relaxed with
        the Smagorinsky rate in the last network step."""
        nu = np.empty(self.N, np.float64)
        self._check(lib().lbm_get_eddy_viscosity(self._ctx, _dp(nu)))
        return nu

    def step_launches(self):
        """Kernel launches one step issues on this context (1, or 2 for the split step)."""
        n = C.c_int32(0)
        self._check(lib().lbm_step_launches(self._ctx, C.byref(n)))
        return n.value

    def probe(self, x, y, z):
        """(u_x, u_y, u_z, rho) of one cell, copied to the host."""
        out = np.empty(4)
        self._check(lib().lbm_probe(self._ctx, int(x), int(y), int(z), _dp(out)))
        return out

    def synchronize(self):
        self._check(lib().lbm_synchronize(self._ctx))

    # -- read-back
    def moments(self):
        rho = np.empty(self.N)
        u = np.empty(3 * self.N)
        self._check(lib().lbm_get_moments(self._ctx, _dp(rho), _dp(u)))
        return rho, u.reshape(3, self.N)

    def populations(self):
        f = np.empty(27 * self.N)
        self._check(lib().lbm_get_populations(self._ctx, _dp(f)))
        return f.reshape(27, self.N)

    def reduce(self, allow_nonfinite=False):
        d = capi.LbmDiag()
        s = lib().lbm_reduce(self._ctx, C.byref(d))
        if s == capi.LBM_ERR_NONFINITE and allow_nonfinite:
            return Diag(d)
        self._check(s)
        return Diag(d)

    def error_evaluation(self):
        e = C.c_double(0)
        self._check(lib().lbm_error_evaluation(self._ctx, C.byref(e)))
        return e.value

    def timeavg_begin(self):
        self._check(lib().lbm_timeavg_begin(self._ctx))

    def timeavg_end(self):
        self._check(lib().lbm_timeavg_end(self._ctx))

    def timeavg_get(self):
        r = np.empty(self.N)
        u = np.empty(3 * self.N)
        uu = np.empty(6 * self.N)
        cnt = C.c_int64(0)
        self._check(lib().lbm_timeavg_get(self._ctx, _dp(r), _dp(u), _dp(uu), C.byref(cnt)))
        return r, u.reshape(3, self.N), uu.reshape(6, self.N), cnt.value

    # -- learned closure
    def load_mlp(self, model):
        """Attach an lb_gb300.les.MlpModel (closure OmegaMLP)."""
        self._check(lib().lbm_mlp_load(self._ctx, C.byref(model.struct())))

    def les_samples(self, width=4):
        """Filtered training samples of the current state (n x 10 float32, see lbm_les_samples)."""
        n = C.c_int64(0)
        self._check(lib().lbm_les_samples(self._ctx, int(width), None, 0, C.byref(n)))
        out = np.zeros((n.value, capi.LBM_MLP_SAMPLE), np.float32)
        if n.value:
            self._check(lib().lbm_les_samples(self._ctx, int(width), out.ctypes.data_as(C.POINTER(C.c_float)),
                                              n.value, C.byref(n)))
        return out

    def checkpoint_save(self, path):
        self._check(lib().lbm_checkpoint_save(self._ctx, str(path).encode()))

    def checkpoint_load(self, path):
        self._check(lib().lbm_checkpoint_load(self._ctx, str(path).encode()))


class SolverTurbulentLES:
    """Reference-shaped driver: SolverTurbulentLES<...>(Constants, Data) with the same method names
    (SolverTurbulentLES.h:106-324).  `constants` is a dict of lattice-unit parameters."""

    def __init__(self, Model=D3Q27, Initialisation=InitializationEquilibriumConstVector,
                 Collision=CollisionCumD3Q27Turbulent2015, Streaming=StreamingAB,
                 BounceBackWall=BounceBackWallHalf, Symmetry=NoSymmetry, Periodic_=NoPeriodic,
                 Inlet=InletVelocityMovingWall, Outlet=OutletDensityInterpolated,
                 Moments=MomentDensityVelocityN27, Turbulence=OmegaLES, Error=ErrorQuadratic,
                 NonDim=NonDimensiolnaliseFactorsVelocity, TimeAvg=MomentTimeAvg, *, constants, data):
        if Model is not D3Q27:
            raise NotImplementedError("only D3Q27 is implemented")
        if Symmetry not in (NoSymmetry, BounceSymmetryHalf):
            raise NotImplementedError(f"symmetry policy {Symmetry.__name__} is not implemented")
        self.C = constants
        self.data = data
        if Initialisation not in (InitializationEquilibriumConstVector, InitializationEquilibriumVariables):
            raise NotImplementedError(f"initialisation policy {Initialisation.__name__} is not implemented")
        self.policies = dict(Collision=Collision, Turbulence=Turbulence, Inlet=Inlet, Outlet=Outlet,
                             Symmetry=Symmetry, Initialisation=Initialisation)
        self.solver = None
        self._converted = False

    def convertToLattice(self, verbose=False):
        """SolverTurbulentLES.h:270-274: converts physical inputs when the constants hold ny_fyz > 0
        (NonDimensiolnaliseFactorsVelocity.nonDimensionalize); lattice-unit constants stay as given."""
        c = self.C
        if not c.get("ny_fyz", 0) > 0:
            return None
        NonDimensiolnaliseFactorsVelocity.nonDimensionalize(c, self.data["flags"].shape[2])
        self._converted = True
        if verbose:
            print(f"Cl {c['Cl']:g} Cu {c['Cu']:g} Ct {c['Ct']:g} Re {c['Re']:g} ny {c['nu']:g} tau {c['tau']:g}")
        return None

    def initializeSimulationData(self, verbose=False):
        """SolverTurbulentLES.h:276-323: plot_every_it, err_every_it and iterations from the physical times
        over Ct (one of plot_every / plot_every_it and of err_every / err_every_it must be given), and the
        probe cell round(x / (BBmax - BBmin + 2 additional / resolution) * n), which must lie inside the
        lattice (the reference's asserts test the reverse of their message, :313-315)."""
        c = self.C
        f = np.float32
        for what in ("plot_every", "err_every"):
            if c.get(what + "_it", -1) == -1:
                if c.get(what, -1) == -1:
                    raise ValueError(f"give {what} or {what}_it")
                c[what + "_it"] = int(np.ceil(f(c[what]) / f(c["Ct"])))
        if c.get("time", -1) >= 0:
            c["iterations"] = int(np.ceil(f(c["time"]) / f(c["Ct"])))
        if c.get("probe_every_it", -1) != -1:
            nz, ny, nx = self.data["flags"].shape
            pad = f(2) * (f(c.get("additional_factor", 0.5)) / f(c.get("resolution_factor", 1.0)))
            lat = []
            for a, n in enumerate((nx, ny, nz)):
                ext = f(c["BBmax"][a]) - f(c["BBmin"][a]) + pad
                v = int(np.round(f(c["ProbeLocation"][a]) / ext * f(n)))
                if not 0 <= v < n:
                    raise ValueError("Probe must be in the domain!")
                lat.append(v)
            c["ProbeLocationLat"] = tuple(lat)
        if verbose:
            print(f"Plotting every {c['plot_every_it']} iterations; {c.get('iterations')} iterations.")

    def initializeSimulation(self, verbose=False):
        c, d = self.C, self.data
        self.solver = Solver(d["flags"].shape[::-1], collision=self.policies["Collision"],
                             turbulence=self.policies["Turbulence"], inlet=self.policies["Inlet"],
                             storage=c.get("storage", "f32"), nu=c["nu"], tau=c.get("tau", 0.0),
                             cles=c.get("CLES", 0.173),
                             periodic=c.get("periodic", (0, 0, 0)), force=c.get("force", (0.0, 0.0, 0.0)),
                             outlet=self.policies["Outlet"],
                             omega_dumping=(c.get("omegaDumpingLow", -1.0), c.get("omegaDumpingHigh", -1.0)))
        self.solver.set_flags(d["flags"])
        inlets, outlets = d.get("inlets", ()), d.get("outlets", ())
        rho0, u0 = c.get("rho0", 1.0), c.get("VelocityInit", (0.0, 0.0, 0.0))
        if self._converted:  # SolverTurbulentLES.h:118, :124; InitializationEquilibriumConstVector.h:79-82
            inlets = NonDimensiolnaliseFactorsVelocity.nonDimensionalizeInlet(inlets, c)
            outlets = NonDimensiolnaliseFactorsVelocity.nonDimensionalizeOutlet(outlets, c)
            f = np.float32
            Cl = f(c["Cl"])
            rho0 = float(f(c.get("rho_fyz", 1.0)) / f(c["Cm"]) * Cl * Cl * Cl)
            u0 = tuple(float(f(v) * f(c["Cu_inverse"])) for v in u0)
        self.solver.set_bc(inlets, outlets)
        if self.policies["Symmetry"] is BounceSymmetryHalf:
            self.solver.set_symmetry(d.get("symmetry", ()))
        if self.policies["Initialisation"] is InitializationEquilibriumVariables:
            from .output import read_variables_vtk
            path = os.path.join(c.get("results_dir") or "results", c["InitFileName"])
            rho, u = read_variables_vtk(path, self.solver.shape)
            self.solver.init_fields(rho, u)
        else:
            self.solver.init_equilibrium(rho0, u0)

    _laminar_loop = False

    def runSimulation(self):
        """The reference's loop (SolverTurbulentLES.h:179-268; SolverLaminar.h:127-204 for the laminar
        solver) in batches of steps between events (step_schedule): the time average over the states after
        step k > iterations - iterationsMomentAvg, the probe, the error (a NaN ends the loop) and, with a
        results_dir, the VTK dumps and probe CSV under their reference names.  Returns [(k, error)]."""
        from . import output
        c = self.C
        it = int(c["iterations"])
        navg = int(c.get("iterationsMomentAvg", 0))
        rdir = c.get("results_dir") or ""
        sched = step_schedule(it, navg, err_every=int(c.get("err_every_it", -1)),
                              probe_every=int(c.get("probe_every_it", -1)),
                              probe_iterations=int(c.get("probe_iterations", -1)),
                              plot_every=int(c.get("plot_every_it", -1)) if rdir else -1, laminar=self._laminar_loop)
        nx, ny, nz = self.solver.shape
        grid = output.Grid((nx, ny, nz), resolution=c.get("resolution_factor", 1.0),
                           additional=c.get("additional_factor", 0.5), bbmin=tuple(c.get("BBmin", (0.0, 0.0, 0.0))))
        conv = {k: c.get(k, 1.0) for k in ("Crho", "Cpressure", "Cu")}
        errors, probes = [], []
        averaging = False
        for begin, n, j, events in sched:
            if begin:
                self.solver.timeavg_begin()
                averaging = True
            self.solver.step(n)
            if "probe" in events:
                sample = self.solver.probe(*c.get("ProbeLocationLat", (0, 0, 0)))
                probes.append(sample)
                if rdir:
                    output.outputerVTK.probeWriteOut(os.path.join(rdir, "probeData.csv"), sample, conv,
                                                     c.get("Ct", 1.0) * int(c["probe_every_it"]))
            if "err" in events:
                e = self.solver.error_evaluation()
                errors.append((j, e))
                if np.isnan(e):
                    break
            if "plot" in events:
                rho, u = self.solver.moments()
                step = j // int(c["plot_every_it"])
                if self._laminar_loop:
                    output.outputerVTK.variablesLatticeVTK(os.path.join(rdir, f"variablesLattice{step}.vtk"), grid,
                                                           rho, u)
                else:
                    output.outputerVTK.variablesVTK(os.path.join(rdir, f"variables.{step}.vtk"), grid, rho, u, conv)
        if averaging:
            self.solver.timeavg_end()
            if rdir:
                rm, um, _, _ = self.solver.timeavg_get()
                output.outputerVTK.variablesTimeAvgVTK(os.path.join(rdir, "variablesTimeAvg.vtk"), grid, rm, um, conv)
        self.probes = probes
        return errors


def step_schedule(it, avg=0, err_every=-1, probe_every=-1, probe_iterations=-1, plot_every=-1, laminar=False):
    """The reference loop's events grouped into runs of steps: [(begin_average, nsteps, j, events)], j the
    0-based index of the batch's last step and events the subset of ("probe", "err", "plot") that the
    reference runs after step j.  A state is averaged when its step k > it - avg (SolverTurbulentLES.h:216),
    probed when k % probe_every == 0 within the last probe_iterations steps (:223; never in the laminar
    loop), the error is taken when k % err_every == 0 and k != 0 (:228), and a dump is written when
    k % plot_every == 0 and k != 0 (:243; from k = 0 on in the laminar loop, SolverLaminar.h:170)."""
    avg_begin = it - avg + 1

    def probe_after(k):
        return not laminar and probe_every > 0 and k % probe_every == 0 and k >= it - probe_iterations

    def err_after(k):
        return err_every > 0 and k % err_every == 0 and k != 0

    def plot_after(k):
        return plot_every > 0 and k % plot_every == 0 and (k != 0 or laminar)

    out, averaging, k = [], False, 0
    while k < it:
        begin = False
        if avg > 0 and not averaging and k >= avg_begin:
            begin = averaging = True
        j = k
        while j < it - 1 and not (probe_after(j) or err_after(j) or plot_after(j)) and \
                not (avg > 0 and not averaging and j + 1 >= avg_begin):
            j += 1
        events = tuple(name for name, f in (("probe", probe_after), ("err", err_after), ("plot", plot_after)) if f(j))
        out.append((begin, j - k + 1, j, events))
        k = j + 1
    return out


class SolverLaminar(SolverTurbulentLES):
    """solvers/SolverLaminar.h:61-237: the same policies without a turbulence model (the step relaxes with
    the global 1/tau) and without the periodic hook, which the reference's laminar loop never calls;
    initializeSimulation runs initializeSimulationData first (:99)."""

    def __init__(self, Model=D3Q27, Initialisation=InitializationEquilibriumConstVector,
                 Collision=CollisionCumD3Q27Laminar, Streaming=StreamingAB, BounceBackWall=BounceBackWallHalf,
                 Symmetry=NoSymmetry, Periodic_=NoPeriodic, Inlet=InletVelocityMovingWall,
                 Outlet=OutletDensityInterpolated, Moments=MomentDensityVelocityN27, Error=ErrorQuadratic,
                 NonDim=NonDimensiolnaliseFactorsVelocity, TimeAvg=MomentTimeAvg, *, constants, data):
        super().__init__(Model, Initialisation, Collision, Streaming, BounceBackWall, Symmetry, Periodic_, Inlet, Outlet,
                         Moments, OmegaNo, Error, NonDim, TimeAvg, constants=constants, data=data)

    _laminar_loop = True

    def initializeSimulation(self, verbose=False):
        self.initializeSimulationData(verbose)
        saved = self.C.get("periodic")
        self.C["periodic"] = (0, 0, 0)
        try:
            super().initializeSimulation(verbose)
        finally:
            if saved is None:
                self.C.pop("periodic")
            else:
                self.C["periodic"] = saved
