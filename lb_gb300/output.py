"""outputerVTK (3D/simulation/src/postprocesors/outputerVTK.h:26-851) over the C ABI writer (lbm_vtk_write,
lbm_probe_csv_append): the reference's legacy VTK field files and probe CSV.

Every writer takes host arrays (rho: N, u: 3N component-major, as Solver.moments() and
Solver.timeavg_get() return them), so a dump costs one device read-back.  `Grid` carries what the
reference keeps in LBMConstants for the header: the lattice size, resolution_factor, additional_factor
and BBmin of the voxelized geometry (lbm_voxelize_off / lbm_mesh_matrix_read return them).  The
conversion factors `conv` (Crho, Cpressure, Cu) are those of NonDimensiolnaliseFactorsVelocity; the lattice
writers use 1.  cs2 = 1/3 (LBMConstants.h:104; MomentPressure.h:32 computes p = rho cs2).
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import capi

CS2 = 1.0 / 3.0


@dataclass
class Grid:
    dims: tuple                  # nx, ny, nz
    resolution: float = 1.0      # resolution_factor
    additional: float = 0.5      # additional_factor (0.5 puts the origin at bbmin)
    bbmin: tuple = (0.0, 0.0, 0.0)


def write_vtk(path, grid, fields, title="LBE variables"):
    """fields: list of (name, array, scale); an array of N values is SCALARS, of 3N (or shape (3, N))
    values VECTORS."""
    nx, ny, nz = (int(d) for d in grid.dims)
    N = nx * ny * nz
    keep, recs = [], []
    for name, arr, scale in fields:
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(-1)
        if a.size not in (N, 3 * N):
            raise ValueError(f"field {name}: {a.size} values for a {nx}x{ny}x{nz} lattice")
        keep.append(a)
        recs.append(capi.LbmVtkField(name.encode(), 1 if a.size == N else 3, a.ctypes.data_as(C.POINTER(C.c_double)),
                                     float(scale)))
    arr = (capi.LbmVtkField * max(len(recs), 1))(*recs)
    dims = np.array([nx, ny, nz], np.int32)
    bb = np.ascontiguousarray(grid.bbmin, dtype=np.float64)
    L = capi.lib()
    st = L.lbm_vtk_write(str(path).encode(), title.encode(), dims.ctypes.data_as(C.POINTER(C.c_int32)),
                         float(grid.resolution), float(grid.additional), bb.ctypes.data_as(C.POINTER(C.c_double)),
                         arr, len(recs))
    if st:
        raise capi.LbmError(st, L.lbm_vtk_last_error().decode())


def read_variables_vtk(path, dims):
    """InitializationEquilibriumVariables' read (InitializationEquilibriumVariables.h:47-113): the first
    LOOKUP_TABLE block as rho and the "VECTORS U double" block as u (3, N), each value parsed as float,
    no conversion factor (restart from a variablesLatticeVTK file)."""
    nx, ny, nz = (int(d) for d in dims)
    N = nx * ny * nz
    rho = np.empty(N, np.float64)
    u = np.empty(3 * N, np.float64)
    d = np.array([nx, ny, nz], np.int32)
    L = capi.lib()
    st = L.lbm_vtk_read_variables(str(path).encode(), d.ctypes.data_as(C.POINTER(C.c_int32)),
                                  rho.ctypes.data_as(C.POINTER(C.c_double)), u.ctypes.data_as(C.POINTER(C.c_double)))
    if st:
        raise capi.LbmError(st, L.lbm_vtk_last_error().decode())
    return rho, u.reshape(3, N)


class outputerVTK:
    """The reference's writer names; paths are used as given (the reference writes under results/)."""

    @staticmethod
    def MeshVTK(path, grid, flags, filename="mesh"):
        """outputerVTK.h:26-56: the flag field as SCALARS object, title "LBE <filename>"."""
        write_vtk(path, grid, [("object", np.asarray(flags).reshape(-1), 1.0)], title=f"LBE {filename}")

    @staticmethod
    def variablesVTK(path, grid, rho, u, conv):
        """outputerVTK.h:59-187: rho*Crho, p*Cpressure (p = rho cs2), U*Cu."""
        rho = np.asarray(rho).reshape(-1)
        write_vtk(path, grid, [("rho", rho, conv["Crho"]), ("p", rho * CS2, conv["Cpressure"]), ("U", u, conv["Cu"])])

    @staticmethod
    def variablesLatticeVTK(path, grid, rho, u):
        """outputerVTK.h:189-316: lattice units, the pressure field named "pressure"."""
        rho = np.asarray(rho).reshape(-1)
        write_vtk(path, grid, [("rho", rho, 1.0), ("pressure", rho * CS2, 1.0), ("U", u, 1.0)])

    @staticmethod
    def variablesTimeAvgVTK(path, grid, rho_mean, u_mean, conv):
        """outputerVTK.h:318-447: the means, pressure rho cs2 Cpressure."""
        rho = np.asarray(rho_mean).reshape(-1)
        write_vtk(path, grid, [("rho", rho, conv["Crho"]), ("pressure", rho * CS2, conv["Cpressure"]),
                               ("U", u_mean, conv["Cu"])])

    @staticmethod
    def variablesTimeAvgLatticeVTK(path, grid, rho_mean, u_mean):
        """outputerVTK.h:449-576."""
        rho = np.asarray(rho_mean).reshape(-1)
        write_vtk(path, grid, [("rho", rho, 1.0), ("pressure", rho * CS2, 1.0), ("U", u_mean, 1.0)])

    @staticmethod
    def omegaVTK(path, grid, omega):
        """outputerVTK.h:578-658: the relaxation rate per cell."""
        write_vtk(path, grid, [("Omega", omega, 1.0)])

    @staticmethod
    def tauVTK(path, grid, omega):
        """outputerVTK.h:742-822: 1/omega per cell as SCALARS Tau."""
        om = np.asarray(omega, dtype=np.float64).reshape(-1)
        tau = (np.float32(1.0) / om.astype(np.float32)).astype(np.float64)
        write_vtk(path, grid, [("Tau", tau, 1.0)])

    @staticmethod
    def distributionFunctionVTK(path, grid, populations, velocity):
        """outputerVTK.h:660-740: one population (reference velocity order) per cell, named as the
        reference names it ("DFunciton_<v>", :690)."""
        f = np.asarray(populations).reshape(27, -1)
        write_vtk(path, grid, [(f"DFunciton_{int(velocity)}", f[int(velocity)], 1.0)])

    @staticmethod
    def probeWriteOut(path, sample, conv, sampling_period):
        """outputerVTK.h:824-851: one line ux,uy,uz,rho,pressure (sample = lbm_probe's u_x, u_y, u_z, rho)."""
        s = np.ascontiguousarray(sample, dtype=np.float64)
        L = capi.lib()
        st = L.lbm_probe_csv_append(str(path).encode(), float(sampling_period), s.ctypes.data_as(C.POINTER(C.c_double)),
                                    float(conv["Cu"]), float(conv["Crho"]), float(conv["Cpressure"]))
        if st:
            raise capi.LbmError(st, L.lbm_vtk_last_error().decode())
