"""geometryMesherBoundary and geometryObjectCuboid (3D/simulation/src/geometry/geometryMesherBoundary.h,
geometryObjectCuboid.h) over the C ABI's host mesher: the wall pass and the cuboid boundary passes with
the reference's method names, building the flag field and the boundary records a case needs.

`constants` carries the sampling frame the reference keeps in LBMConstants: dimX_int / dimY_int /
dimZ_int (or the flag array's shape), resolution_factor, additional_factor and BBmin.  `data["flags"]` is
the flag field [z, y, x] (int32, changed in place, as the reference changes meshFluidHost); the passes
collect records, and compileBoundaryArray* put them into data["inlets"], ["outlets"], ["symmetry"],
["periodic"] for Solver.set_bc / set_symmetry.  geometryHandlerOFF and geometryMesherOFF are the
preprocessor's OFF reader and polyhedron mesher (preprocess.cpp:60-72) over lbm_voxelize_off.
"""
import ctypes as C
import math

import numpy as np

from . import capi


class geometryObjectCuboid:
    """The axis box spanned by three corners X1, X2, X3, closed on every face; id is the negative flag
    its cells get (-1 inlet, -2 outlet or symmetry, -3 periodic)."""

    def __init__(self, X1, X2, X3, id):
        self.X = (tuple(map(float, X1)), tuple(map(float, X2)), tuple(map(float, X3)))
        self.id = int(id)

    def isInside(self, p):
        return all(min(x[a] for x in self.X) <= p[a] <= max(x[a] for x in self.X) for a in range(3))

    def struct(self):
        c = capi.LbmCuboid()
        for a in range(3):
            c.x1[a], c.x2[a], c.x3[a] = self.X[0][a], self.X[1][a], self.X[2][a]
        c.id = self.id
        return c


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


class geometryMesherBoundary:
    def __init__(self, constants, data):
        self.C = constants
        self.data = data
        f = data["flags"]
        if f.dtype != np.int32 or not f.flags.c_contiguous:
            raise ValueError("data['flags'] must be a C-contiguous int32 array [z, y, x]")
        self.inlets, self.outlets, self.symmetry, self.periodic = [], [], [], []

    # -- frame and capacity
    def _frame(self):
        nz, ny, nx = self.data["flags"].shape
        fr = capi.LbmMeshFrame()
        fr.dims[0], fr.dims[1], fr.dims[2] = nx, ny, nz
        fr.resolution_factor = float(self.C.get("resolution_factor", 1.0))
        fr.additional_factor = float(self.C.get("additional_factor", 0.5))
        bb = self.C.get("BBmin", (0.0, 0.0, 0.0))
        for a in range(3):
            fr.bbmin[a] = float(bb[a])
        return fr

    def _bound(self, cuboid):
        """An upper bound on the cells whose centre lies in the cuboid (its index box widened by one)."""
        fr = self._frame()
        n = 1
        for a in range(3):
            lo = min(x[a] for x in cuboid.X)
            hi = max(x[a] for x in cuboid.X)
            res, add, bb = fr.resolution_factor, fr.additional_factor, fr.bbmin[a]
            i0 = math.floor((lo - bb) * res + add - 0.5) - 1
            i1 = math.ceil((hi - bb) * res + add - 0.5) + 1
            n *= max(0, min(fr.dims[a] - 1, i1) - max(0, i0) + 1)
        return n

    def _run(self, fn, rtype, store, cuboid, *args):
        cap = len(store) + self._bound(cuboid)
        arr = (rtype * max(cap, 1))(*store)
        n = C.c_int64(len(store))
        fr = self._frame()
        cub = cuboid.struct()
        flags = self.data["flags"]
        L = capi.lib()
        st = getattr(L, fn)(C.byref(fr), flags.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(cub), *args, arr, cap,
                            C.byref(n))
        if st:
            raise capi.LbmError(st, L.lbm_mesher_last_error().decode())
        added = n.value - len(store)
        store[:] = [arr[i] for i in range(n.value)]
        return added

    # -- passes (geometryMesherBoundary.h:47-484)
    def meshingBoundaryWall(self, verbose=False):
        """:439-484: every fluid cell gets 1 + the number of solid cells among its 26 neighbours."""
        f = self.data["flags"]
        nz, ny, nx = f.shape
        capi.check(capi.lib().lbm_mesher_wall_pass(f.ctypes.data_as(C.POINTER(C.c_int32)), nx, ny, nz))

    def meshingBoundaryConditionInletUniform(self, cuboid, normal_out, velocity_in, verbose=False):
        n = self._run("lbm_mesher_inlet_uniform", capi.LbmBcInlet, self.inlets, cuboid, _f3(normal_out),
                      _f3(velocity_in))
        if verbose:
            print(f"Meshed cuboid id {cuboid.id} as Inlet: {n} nodes")
        return n

    def meshingBoundaryConditionInletParaboloidCircle(self, cuboid, inletCenter, inletRadius, normal_out,
                                                      mean_velocity_in, verbose=False):
        c = (C.c_double * 3)(*[float(x) for x in inletCenter])
        n = self._run("lbm_mesher_inlet_paraboloid_circle", capi.LbmBcInlet, self.inlets, cuboid, c,
                      float(inletRadius), _f3(normal_out), float(mean_velocity_in))
        if verbose:
            print(f"Meshed cuboid id {cuboid.id} as Inlet: {n} nodes")
        return n

    def meshingBoundaryConditionInletParaboloidRectangle(self, cuboid, inletCenter, inletDimX, inletDimY, inletDimZ,
                                                         normal_out, mean_velocity_in, verbose=False):
        """Returns the inlet dimensions as the pass leaves them (1 along the normal: the reference writes
        them back through its by-reference arguments)."""
        c = (C.c_double * 3)(*[float(x) for x in inletCenter])
        dims = _f3((inletDimX, inletDimY, inletDimZ))
        n = self._run("lbm_mesher_inlet_paraboloid_rectangle", capi.LbmBcInlet, self.inlets, cuboid, c, dims,
                      _f3(normal_out), float(mean_velocity_in))
        if verbose:
            print(f"Meshed cuboid id {cuboid.id} as Inlet: {n} nodes")
        return tuple(dims)

    def meshingBoundaryConditionOutlet(self, cuboid, normal_out, density, verbose=False):
        n = self._run("lbm_mesher_outlet", capi.LbmBcOutlet, self.outlets, cuboid, _f3(normal_out), float(density))
        if verbose:
            print(f"Meshed cuboid id {cuboid.id} as outlet: {n} nodes")
        return n

    def meshingBoundaryConditionSymmetry(self, cuboid, normal_out, verbose=False):
        n = self._run("lbm_mesher_symmetry", capi.LbmBcSymmetry, self.symmetry, cuboid, _f3(normal_out))
        if verbose:
            print(f"Meshed cuboid id {cuboid.id} as Symmetry: {n} nodes")
        return n

    def meshingBoundaryConditionPeriodic(self, cuboid, normal_out, periodicIndex_, verbose=False):
        n = self._run("lbm_mesher_periodic", capi.LbmBcPeriodic, self.periodic, cuboid, _f3(normal_out),
                      int(periodicIndex_))
        if verbose:
            print(f"Meshed cuboid id {cuboid.id} as Periodic: {n} nodes")
        return n

    # -- record lists (:486-603)
    def compileBoundaryArrayInlets(self, verbose=False):
        self.data["inlets"] = list(self.inlets)

    def compileBoundaryArrayOutlets(self, verbose=False):
        self.data["outlets"] = list(self.outlets)

    def compileBoundaryArraySymmetry(self, verbose=False):
        self.data["symmetry"] = list(self.symmetry)

    def compileBoundaryArrayPeriodic(self, verbose=False):
        """Records for reference tooling; the kernels wrap periodic axes by index (Solver periodic=)."""
        self.data["periodic_records"] = list(self.periodic)

    def compileBoundaryArrayWall(self, verbose=False):
        """:534-560: the wall nodes (flag > 2 after the wall pass) that no boundary pass took (flag < 0
        erased); the kernels find wall links from the flags themselves, so this list is informational."""
        f = self.data["flags"]
        z, y, x = np.nonzero(f > 2)
        self.data["walls"] = np.stack([x, y, z], axis=1).astype(np.int32)

    def arrayTransfer(self, verbose=False):
        return None  # the Solver uploads flags and records itself


class geometryHandlerOFF:
    """preprocess/src/geometry/geometryHandlerOFF.h: reads the OFF/NOFF file and its bounding box (float, as
    LBMConstants keeps it) through lbm_voxelize_off's size query (host code, no GPU)."""

    def __init__(self):
        self.path = None
        self.bbox = None
        self.dims = None

    def polyhedronFromFile(self, constants, verbose=False):
        self.path = str(constants["file_name"])
        dims = np.zeros(3, np.int32)
        bbox = np.zeros(6, np.float64)
        out = np.asarray(constants.get("point_outside", (-1.0, -1.0, -1.0)), np.float64)
        st = capi.lib().lbm_voxelize_off(self.path.encode(), float(constants["resolution_factor"]),
                                         float(constants["additional_factor"]), out.ctypes.data_as(C.POINTER(C.c_double)),
                                         None, dims.ctypes.data_as(C.POINTER(C.c_int32)),
                                         bbox.ctypes.data_as(C.POINTER(C.c_double)), 0)
        if st:
            raise capi.LbmError(st, f"cannot read the OFF file {self.path}")
        self.bbox, self.dims = bbox, tuple(int(d) for d in dims)

    def polyhedronBbox(self, verbose=False):
        return None  # the bounding box comes with the read

    def writeToConstants(self, constants):
        constants["BBmin"] = tuple(float(v) for v in self.bbox[:3])
        constants["BBmax"] = tuple(float(v) for v in self.bbox[3:])


class geometryMesherOFF:
    """preprocess/src/geometry/geometryMesherOFF.h:45-112: the lattice from the bounding box, then 1 inside
    the polyhedron and 0 outside at every cell centre (the GPU voxelizer)."""

    def __init__(self, constants, data):
        self.C = constants
        self.data = data

    def initialization(self, verbose=False):
        f = np.float32
        dims = []
        for a in range(3):
            ext = f(self.C["BBmax"][a]) - f(self.C["BBmin"][a])
            dims.append(int(np.ceil(ext * f(self.C["resolution_factor"]) + f(2) * f(self.C["additional_factor"]))))
        self.C["dimX_int"], self.C["dimY_int"], self.C["dimZ_int"] = dims
        self.data["flags"] = np.zeros(dims[::-1], np.int32)

    def meshingPolyhedron(self, handler, point_outside, verbose=False):
        nx, ny, nz = self.C["dimX_int"], self.C["dimY_int"], self.C["dimZ_int"]
        if handler.dims != (nx, ny, nz):
            raise ValueError("the lattice does not match the polyhedron's bounding box")
        flags = np.zeros((nz, ny, nx), np.int32)
        dims = np.zeros(3, np.int32)
        bbox = np.zeros(6, np.float64)
        out = np.asarray(point_outside, np.float64)
        st = capi.lib().lbm_voxelize_off(handler.path.encode(), float(self.C["resolution_factor"]),
                                         float(self.C["additional_factor"]), out.ctypes.data_as(C.POINTER(C.c_double)),
                                         flags.ctypes.data_as(C.POINTER(C.c_int32)),
                                         dims.ctypes.data_as(C.POINTER(C.c_int32)),
                                         bbox.ctypes.data_as(C.POINTER(C.c_double)), int(self.C.get("device", 0)))
        if st:
            raise capi.LbmError(st, f"lbm_voxelize_off failed on {handler.path}")
        self.data["flags"] = flags


def fold_periodic(flags, periodic_records, inlets=(), outlets=(), symmetry=()):
    """A lattice made periodic the reference's way (Periodic.h: two planes of -3 nodes per axis whose
    records point at each other, each copying the other's entering populations) as the index-wrapped
    lattice the kernels run.  With the pair at planes p < q of axis a, planes p .. q-1 are kept (plane q
    repeats plane p) and axis a wraps; the -3 flags become plain fluid (1) and the records move with the
    planes.  Returns dict(flags, periodic, offset, inlets, outlets, symmetry); records on dropped planes
    are dropped.  The ghost-plane and index-wrap forms step identically (tested on the oracle)."""
    f = np.ascontiguousarray(flags, dtype=np.int32)
    nz, ny, nx = f.shape
    n = (nx, ny, nz)
    pairs = {}
    for r in periodic_records:
        nrm = tuple(int(round(v)) for v in r.normal)
        axes = [a for a in range(3) if nrm[a] != 0]
        if len(axes) != 1:
            raise ValueError("periodic record with a normal off the axes")
        a = axes[0]
        plane = (r.vertex.x, r.vertex.y, r.vertex.z)[a]
        pairs.setdefault(a, set()).add((plane, int(r.periodic_index)))
    lo, hi, periodic = [0, 0, 0], list(n), [0, 0, 0]
    for a, ps in pairs.items():
        if len(ps) != 2:
            raise ValueError(f"axis {a}: expected two periodic planes pointing at each other, found {sorted(ps)}")
        (p, pi), (q, qi) = sorted(ps)
        if pi != q or qi != p or q <= p:
            raise ValueError(f"axis {a}: planes {p} and {q} do not point at each other ({pi}, {qi})")
        lo[a], hi[a], periodic[a] = p, q, 1
    out = f[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]].copy()
    out[out == -3] = 1

    def move(records, make):
        kept = []
        for r in records:
            v = (r.vertex.x, r.vertex.y, r.vertex.z)
            if all(lo[a] <= v[a] < hi[a] for a in range(3)):
                kept.append(make(r, [v[a] - lo[a] for a in range(3)]))
        return kept

    return dict(flags=out, periodic=tuple(periodic), offset=tuple(lo),
                inlets=move(inlets, lambda r, v: capi.make_inlet(*v, tuple(r.normal), tuple(r.velocity), r.regular)),
                outlets=move(outlets, lambda r, v: capi.make_outlet(*v, tuple(r.normal), r.density, r.regular)),
                symmetry=move(symmetry, lambda r, v: capi.make_symmetry(*v, tuple(r.normal), r.regular)))
