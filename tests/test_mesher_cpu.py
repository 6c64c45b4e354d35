"""The cuboid boundary passes of the host mesher (geometryMesherBoundary.h:47-437, geometryObjectCuboid.h:20-38)
on the CPU, against the passes restated here in numpy with the reference's float/double steps: which cells
a cuboid takes (centre test, flag condition, loop order), the flags they get, and every record field."""
import ctypes as C

import numpy as np
import pytest

from lb_gb300 import capi
from lb_gb300.mesher import geometryMesherBoundary, geometryObjectCuboid

F = np.float32
# a frame where the float rounding of the look coordinate matters: resolution 2.5, additional 1.5
FRAME = dict(resolution_factor=2.5, additional_factor=1.5, BBmin=(-0.3, 0.1, 0.7))
SHAPE = (7, 9, 14)  # z, y, x


def look(frame, idx, axis, as_float):
    v = (idx + 0.5 - float(F(frame["additional_factor"]))) / float(F(frame["resolution_factor"])) + \
        float(F(frame["BBmin"][axis]))
    return float(F(v)) if as_float else v


def taken(frame, flags, cub, inlet):
    """(index, z, y, x) of the cells a pass takes, in the reference's k, j, i order."""
    out = []
    nz, ny, nx = flags.shape
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                fl = flags[k, j, i]
                if (fl <= 0) if inlet else (fl == 0):
                    continue
                p = [look(frame, i, 0, inlet), look(frame, j, 1, inlet), look(frame, k, 2, inlet)]
                if cub.isInside(p):
                    out.append((k, j, i))
    return out


def channel_flags():
    """Solid walls at y = 0 and y = ny-1 and a solid block, then the wall pass."""
    f = np.ones(SHAPE, np.int32)
    f[:, 0, :] = 0
    f[:, -1, :] = 0
    f[2:4, 3:5, 6:8] = 0
    m = geometryMesherBoundary(dict(FRAME), {"flags": f})
    m.meshingBoundaryWall()
    return f


def x_of(i):
    return (i + 0.5 - 1.5) / 2.5 - 0.3


def test_plane_passes_match_the_restatement(built_lib):
    f = channel_flags()
    f0 = f.copy()
    m = geometryMesherBoundary(dict(FRAME), {"flags": f})
    # a plane through the cell centres of x = 0 and one of x = nx-1, spanning all of y and z
    inlet = geometryObjectCuboid((x_of(0) - 0.01, -1, -1), (x_of(0) + 0.01, 10, 10), (x_of(0), 10, -1), -1)
    outlet = geometryObjectCuboid((x_of(13) - 0.01, -1, -1), (x_of(13) + 0.01, 10, 10), (x_of(13), -1, 10), -2)
    sym = geometryObjectCuboid((-5, (7 + 0.5 - 1.5) / 2.5 + 0.1 - 0.01, -5), (10, 3.0, 10), (0, 3.0, 0), -2)
    per = geometryObjectCuboid((-5, -5, (0 + 0.5 - 1.5) / 2.5 + 0.7 - 0.01), (10, 10, 0.31), (0, 0, 0.31), -3)
    ref = f0.copy()
    expect_in = taken(FRAME, ref, inlet, True)
    n_in = m.meshingBoundaryConditionInletUniform(inlet, (-1, 0, 0), (0.05, 0.0, 0.001))
    for k, j, i in expect_in:
        ref[k, j, i] = -1
    expect_out = taken(FRAME, ref, outlet, False)
    m.meshingBoundaryConditionOutlet(outlet, (1, 0, 0), 1.25)
    out_regular = [int(ref[k, j, i] == 10) for k, j, i in expect_out]
    for k, j, i in expect_out:
        ref[k, j, i] = -2
    expect_sym = taken(FRAME, ref, sym, False)
    m.meshingBoundaryConditionSymmetry(sym, (0, 1, 0))
    sym_regular = [int(ref[k, j, i] == 10) for k, j, i in expect_sym]
    for k, j, i in expect_sym:
        ref[k, j, i] = -2
    expect_per = taken(FRAME, ref, per, False)
    m.meshingBoundaryConditionPeriodic(per, (0, 0, -1), 5)
    per_regular = [int(ref[k, j, i] == 10) for k, j, i in expect_per]
    for k, j, i in expect_per:
        ref[k, j, i] = -3
    assert np.array_equal(f, ref)
    assert n_in == len(expect_in) == 7 * 7  # y = 1..7 fluid, all z
    assert [(r.vertex.z, r.vertex.y, r.vertex.x) for r in m.inlets] == expect_in
    assert all(r.regular == int(f0[r.vertex.z, r.vertex.y, r.vertex.x] <= 10) for r in m.inlets)
    assert all(tuple(r.velocity) == (F(0.05), 0.0, F(0.001)) and tuple(r.normal) == (-1, 0, 0) for r in m.inlets)
    assert [(r.vertex.z, r.vertex.y, r.vertex.x) for r in m.outlets] == expect_out
    assert [r.regular for r in m.outlets] == out_regular
    assert all(r.density == 1.25 for r in m.outlets)
    assert [(r.vertex.z, r.vertex.y, r.vertex.x) for r in m.symmetry] == expect_sym and expect_sym
    assert [r.regular for r in m.symmetry] == sym_regular and 1 in sym_regular and 0 in sym_regular
    assert [(r.vertex.z, r.vertex.y, r.vertex.x) for r in m.periodic] == expect_per and expect_per
    assert [r.regular for r in m.periodic] == per_regular
    assert all(r.periodic_index == 5 for r in m.periodic)
    m.compileBoundaryArrayInlets()
    m.compileBoundaryArrayOutlets()
    m.compileBoundaryArrayWall()
    assert len(m.data["inlets"]) == n_in and len(m.data["outlets"]) == len(expect_out)
    assert all(f[z, y, x] > 2 for x, y, z in m.data["walls"])


def test_uniform_inlet_guard_and_capacity(built_lib):
    f = channel_flags()
    m = geometryMesherBoundary(dict(FRAME), {"flags": f})
    cub = geometryObjectCuboid((-10, -10, -10), (10, 10, 10), (0, 0, 0), -1)
    with pytest.raises(capi.LbmError) as e:
        m.meshingBoundaryConditionInletUniform(cub, (-1, 0, 0), (0.0, 0.0, 0.0))
    assert e.value.status == capi.LBM_ERR_INVALID
    # too little room: nothing written
    fr = m._frame()
    c = cub.struct()
    n = C.c_int64(0)
    rec = (capi.LbmBcInlet * 3)()
    before = f.copy()
    st = capi.lib().lbm_mesher_inlet_uniform(C.byref(fr), f.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(c),
                                             (C.c_float * 3)(-1, 0, 0), (C.c_float * 3)(0.1, 0, 0), rec, 3, C.byref(n))
    assert st == capi.LBM_ERR_INVALID and n.value == 0 and np.array_equal(f, before)


def test_paraboloid_inlets_match_the_restatement(built_lib):
    f = channel_flags()
    frame = dict(FRAME)
    m = geometryMesherBoundary(frame, {"flags": f})
    x0 = x_of(0)
    cub = geometryObjectCuboid((x0 - 0.01, -1, -1), (x0 + 0.01, 10, 10), (x0, 10, -1), -1)
    centre = (x0, 1.5, 2.1)
    radius, umean = 1.3, 0.04
    m.meshingBoundaryConditionInletParaboloidCircle(cub, centre, radius, (-1, 0, 0), umean)
    hit = 0
    for r in m.inlets:
        p = [look(frame, r.vertex.x, 0, True), look(frame, r.vertex.y, 1, True), look(frame, r.vertex.z, 2, True)]
        d = F(np.sqrt(sum((p[a] - centre[a]) ** 2 for a in range(3))))
        v = F(0)
        if d <= F(radius):
            v = F(float(F(3) * F(umean)) * (1.0 - float(F(d / F(radius))) ** 2))
            v = max(v, F(0))
            hit += 1
        assert r.velocity[0] == -v * F(-1) and r.velocity[1] == 0 and r.velocity[2] == 0
    assert 0 < hit < len(m.inlets)

    f2 = channel_flags()
    m2 = geometryMesherBoundary(frame, {"flags": f2})
    dims = (1.0, 2.8, 2.6)
    ctr = (x0, 1.5, 1.9)
    left = m2.meshingBoundaryConditionInletParaboloidRectangle(cub, ctr, *dims, (-1, 0, 0), umean)
    assert left == (1.0, F(2.8), F(2.6))
    D = [F(1.0), F(2.8), F(2.6)]
    k = D[0] * D[1] * D[2] * D[0] * D[1] * D[2] / F(16)
    for r in m2.inlets:
        p = [look(frame, r.vertex.x, 0, True), look(frame, r.vertex.y, 1, True), look(frame, r.vertex.z, 2, True)]
        part = [F(1.0)]
        for a in (1, 2):
            s = F(p[a] - (ctr[a] - float(D[a] / F(2))))
            part.append(s * (D[a] - s))
        v = F(2) * F(umean) * part[0] * part[1] * part[2] / k
        v = max(v, F(0))
        assert r.velocity[0] == v, (r.vertex.y, r.vertex.z, r.velocity[0], v)
    assert max(r.velocity[0] for r in m2.inlets) > 0


def test_cpp_mesher_equals_python(built_lib):
    """geometryMesherBoundary of the C++ mirror (include/lbm_solver.hpp) on the same case: the same flags and
    records as the Python mirror."""
    import os
    import subprocess
    import tempfile
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    x0, x13 = x_of(0), x_of(13)
    src = r'''
#include <cstdio>
#include "lbm_solver.hpp"
using namespace lbm_gb300;
int main() {
    LBMConstants C; LBMData D;
    C.dimX_int = 14; C.dimY_int = 9; C.dimZ_int = 7;
    C.resolution_factor = 2.5; C.additional_factor = 1.5; C.BBmin[0] = -0.3; C.BBmin[1] = 0.1; C.BBmin[2] = 0.7;
    D.meshFluid.assign(14 * 9 * 7, 1);
    for (int k = 0; k < 7; k++) for (int j = 0; j < 9; j++) for (int i = 0; i < 14; i++) {
        const bool solid = j == 0 || j == 8 || (k >= 2 && k < 4 && j >= 3 && j < 5 && i >= 6 && i < 8);
        if (solid) D.meshFluid[(k * 9 + j) * 14 + i] = 0;
    }
    geometryMesherBoundary M(C, D);
    M.meshingBoundaryWall(false);
    const double a1[3] = {%r, -1, -1}, a2[3] = {%r, 10, 10}, a3[3] = {%r, 10, -1};
    const double b1[3] = {%r, -1, -1}, b2[3] = {%r, 10, 10}, b3[3] = {%r, -1, 10};
    geometryObjectCuboid inlet(a1, a2, a3, -1), outlet(b1, b2, b3, -2);
    const float nin[3] = {-1, 0, 0}, nout[3] = {1, 0, 0};
    const double centre[3] = {%r, 1.5, 2.1};
    M.meshingBoundaryConditionInletParaboloidCircle(inlet, centre, 1.3f, nin, 0.04f, false);
    M.meshingBoundaryConditionOutlet(outlet, nout, 1.25f, false);
    long long s = 0;
    for (size_t q = 0; q < D.meshFluid.size(); q++) s += (long long)D.meshFluid[q] * (long long)(q + 1);
    std::printf("%%lld %%zu %%zu\n", s, D.meshBoundaryInlet.size(), D.meshBoundaryOutlet.size());
    for (auto& r : D.meshBoundaryInlet) std::printf("%%d %%d %%d %%.9g %%d\n", r.vertex.x, r.vertex.y, r.vertex.z, r.velocity[0], r.regular);
    for (auto& r : D.meshBoundaryOutlet) std::printf("%%d %%d %%d %%d\n", r.vertex.x, r.vertex.y, r.vertex.z, r.regular);
    return 0;
}
''' % (x0 - 0.01, x0 + 0.01, x0, x13 - 0.01, x13 + 0.01, x13, x0)
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "t.cpp")
        exe = os.path.join(d, "t")
        with open(p, "w") as fh:
            fh.write(src)
        lib = os.path.join(root, "lb_gb300")
        r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(root, "include"), p, "-L", lib, "-llbm_gb300",
                            "-Wl,-rpath," + lib, "-o", exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines()
    f = channel_flags()
    m = geometryMesherBoundary(dict(FRAME), {"flags": f})
    inlet = geometryObjectCuboid((x0 - 0.01, -1, -1), (x0 + 0.01, 10, 10), (x0, 10, -1), -1)
    outlet = geometryObjectCuboid((x13 - 0.01, -1, -1), (x13 + 0.01, 10, 10), (x13, -1, 10), -2)
    m.meshingBoundaryConditionInletParaboloidCircle(inlet, (x0, 1.5, 2.1), 1.3, (-1, 0, 0), 0.04)
    m.meshingBoundaryConditionOutlet(outlet, (1, 0, 0), 1.25)
    s = int((f.reshape(-1).astype(np.int64) * np.arange(1, f.size + 1)).sum())
    want = ["%d %d %d" % (s, len(m.inlets), len(m.outlets))]
    want += ["%d %d %d %.9g %d" % (r.vertex.x, r.vertex.y, r.vertex.z, r.velocity[0], r.regular) for r in m.inlets]
    want += ["%d %d %d %d" % (r.vertex.x, r.vertex.y, r.vertex.z, r.regular) for r in m.outlets]
    assert out == want


def test_off_handler_and_mesher_size_the_golden_lattice(built_lib):
    """geometryHandlerOFF / geometryMesherOFF of both mirrors on the reference's BackwardStepLaminar.off:
    the bounding box and the lattice dimensions of the golden mesh-matrix file (the flags themselves are
    the GPU voxelizer's, checked bit for bit on the GPU)."""
    import os
    import subprocess
    import tempfile
    from lb_gb300.mesher import geometryHandlerOFF, geometryMesherOFF
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    gold = os.path.join(root, "tests", "golden")
    g = np.load(os.path.join(gold, "backward_step_laminar.npz"))
    off = os.path.join(gold, "BackwardStepLaminar.off")
    c = dict(file_name=off, resolution_factor=float(g["resolution"]), additional_factor=float(g["additional"]))
    h = geometryHandlerOFF()
    h.polyhedronFromFile(c)
    h.polyhedronBbox()
    h.writeToConstants(c)
    d = {}
    geometryMesherOFF(c, d).initialization()
    assert (c["dimX_int"], c["dimY_int"], c["dimZ_int"]) == tuple(int(v) for v in g["dims"]) == h.dims
    assert d["flags"].shape == tuple(int(v) for v in g["dims"][::-1])
    assert np.allclose(c["BBmin"], g["bbmin"], rtol=0, atol=1e-6) and np.allclose(c["BBmax"], g["bbmax"], rtol=0, atol=1e-6)
    src = r'''
#include <cstdio>
#include "lbm_solver.hpp"
using namespace lbm_gb300;
int main(int argc, char** argv) {
    LBMConstants C; LBMData D;
    C.file_name = argv[1]; C.resolution_factor = %r; C.additional_factor = %r;
    geometryHandlerOFF H;
    H.polyhedronFromFile(C, false);
    H.writeToConstants(C);
    geometryMesherOFF M(C, D);
    M.initialization(false);
    std::printf("%%d %%d %%d %%zu %%.9g %%.9g\n", C.dimX_int, C.dimY_int, C.dimZ_int, D.meshFluid.size(), C.BBmin[0], C.BBmax[2]);
    return 0;
}
''' % (float(g["resolution"]), float(g["additional"]))
    with tempfile.TemporaryDirectory() as t:
        p = os.path.join(t, "t.cpp")
        exe = os.path.join(t, "t")
        with open(p, "w") as fh:
            fh.write(src)
        lib = os.path.join(root, "lb_gb300")
        r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(root, "include"), p, "-L", lib, "-llbm_gb300",
                            "-Wl,-rpath," + lib, "-o", exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out = subprocess.run([exe, off], capture_output=True, text=True, check=True).stdout.split()
    n = [int(v) for v in g["dims"]]
    assert out[:4] == [str(n[0]), str(n[1]), str(n[2]), str(n[0] * n[1] * n[2])]
    assert float(out[4]) == float("%.9g" % c["BBmin"][0]) and float(out[5]) == float("%.9g" % c["BBmax"][2])


def test_fold_periodic_steps_like_the_ghost_planes(built_lib, oracle_lib):
    """A lattice made periodic in x the reference's way (solid planes 0 and L+2, the mesher's periodic
    pass on planes 1 and L+1 pointing at each other, as main.cu:176-177 builds it) folded by
    fold_periodic steps like the ghost-plane form on the oracle (Periodic.h:43-138) to 1e-13."""
    from oracle import oracle as O
    from lb_gb300.mesher import fold_periodic
    L, ny, nz = 9, 5, 4
    X = L + 3
    f = np.ones((nz, ny, X), np.int32)
    f[:, :, 0] = 0
    f[:, :, -1] = 0
    frame = dict(resolution_factor=1.0, additional_factor=0.5, BBmin=(0.0, 0.0, 0.0))  # centres at integers
    m = geometryMesherBoundary(frame, {"flags": f})
    m.meshingBoundaryWall()
    m.meshingBoundaryConditionPeriodic(geometryObjectCuboid((0.9, -1, -1), (1.1, 99, 99), (1.0, 99, -1), -3),
                                       (-1, 0, 0), L + 1)
    m.meshingBoundaryConditionPeriodic(geometryObjectCuboid((L + 0.9, -1, -1), (L + 1.1, 99, 99), (L + 1, -1, 99), -3),
                                       (1, 0, 0), 1)
    assert len(m.periodic) == 2 * ny * nz
    fo = fold_periodic(f, m.periodic)
    assert fo["periodic"] == (1, 0, 0) and fo["offset"] == (1, 0, 0)
    assert np.array_equal(fo["flags"], np.ones((nz, ny, L), np.int32))
    rng = np.random.default_rng(11)
    rho = 1 + 0.01 * rng.standard_normal(L * ny * nz)
    u = 0.03 * rng.standard_normal((3, L * ny * nz))
    kw = dict(nu=0.02, collision=capi.LBM_COLLISION_CUMULANT2015, closure=capi.LBM_CLOSURE_SMAGORINSKY)
    a = O.OracleSim(capi.make_config(L, ny, nz, periodic=(1, 1, 1), **kw), 64)
    a.set_flags(fo["flags"])
    a.set_bc()
    a.init_fields(rho, u)
    b = O.OracleSim(capi.make_config(X, ny, nz, periodic=(0, 1, 1), **kw), 64)
    b.set_flags(f)
    b.set_bc()
    b.set_periodic_list([[r.vertex.x, r.vertex.y, r.vertex.z, *[int(v) for v in r.normal], r.periodic_index, r.regular]
                         for r in m.periodic])
    r3, u3 = rho.reshape(nz, ny, L), u.reshape(3, nz, ny, L)
    rg, ug = np.ones((nz, ny, X)), np.zeros((3, nz, ny, X))
    for p in range(1, L + 2):  # ghost plane p holds folded plane (p - 1) mod L
        rg[:, :, p] = r3[:, :, (p - 1) % L]
        ug[:, :, :, p] = u3[:, :, :, (p - 1) % L]
    b.init_fields(rg.reshape(-1), ug.reshape(3, -1))
    for _ in range(5):
        a.step(1)
        b.step(1)
        ra, ua = a.moments()
        rb, ub = b.moments()
        assert np.abs(ra.reshape(nz, ny, L) - rb.reshape(nz, ny, X)[:, :, 1:L + 1]).max() < 1e-13
        assert np.abs(ua.reshape(3, nz, ny, L) - ub.reshape(3, nz, ny, X)[:, :, :, 1:L + 1]).max() < 1e-13
    with pytest.raises(ValueError):
        fold_periodic(f, m.periodic[: ny * nz])  # one plane without its partner


def test_cpp_fold_periodic_equals_python(built_lib):
    import os
    import subprocess
    import tempfile
    from lb_gb300.mesher import fold_periodic
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = r'''
#include <cstdio>
#include "lbm_solver.hpp"
using namespace lbm_gb300;
int main() {
    LBMConstants C; LBMData D;
    C.dimX_int = 12; C.dimY_int = 5; C.dimZ_int = 4;
    D.meshFluid.assign(12 * 5 * 4, 1);
    for (int k = 0; k < 4; k++) for (int j = 0; j < 5; j++) {
        D.meshFluid[(k * 5 + j) * 12 + 0] = 0; D.meshFluid[(k * 5 + j) * 12 + 11] = 0;
        if (j == 2) D.meshFluid[(k * 5 + j) * 12 + 6] = 0;
    }
    geometryMesherBoundary M(C, D);
    M.meshingBoundaryWall(false);
    const double a1[3] = {0.9, -1, -1}, a2[3] = {1.1, 99, 99}, a3[3] = {1.0, 99, -1};
    const double b1[3] = {9.9, -1, -1}, b2[3] = {10.1, 99, 99}, b3[3] = {10.0, -1, 99};
    const double c1[3] = {4.9, -1, -1}, c2[3] = {5.1, 99, 99}, c3[3] = {5.0, -1, 99};
    const float nm[3] = {-1, 0, 0}, np_[3] = {1, 0, 0}, vin[3] = {0.04f, 0.f, 0.001f};
    C.resolution_factor = 1.0; C.additional_factor = 0.5;
    M.meshingBoundaryConditionPeriodic(geometryObjectCuboid(a1, a2, a3, -3), nm, 10, false);
    M.meshingBoundaryConditionPeriodic(geometryObjectCuboid(b1, b2, b3, -3), np_, 1, false);
    M.meshingBoundaryConditionInletUniform(geometryObjectCuboid(c1, c2, c3, -1), nm, vin, false);
    foldPeriodic(C, D);
    long long s = 0;
    for (size_t q = 0; q < D.meshFluid.size(); q++) s += (long long)D.meshFluid[q] * (long long)(q + 1);
    std::printf("%d %d %d %d %d %d %lld %zu", C.dimX_int, C.dimY_int, C.dimZ_int, C.periodic[0], C.periodic[1],
                C.periodic[2], s, D.meshBoundaryInlet.size());
    for (auto& r : D.meshBoundaryInlet) std::printf(" %d/%d/%d", r.vertex.x, r.vertex.y, r.vertex.z);
    std::printf("\n");
    return 0;
}
'''
    with tempfile.TemporaryDirectory() as t:
        p = os.path.join(t, "t.cpp")
        exe = os.path.join(t, "t")
        with open(p, "w") as fh:
            fh.write(src)
        lib = os.path.join(root, "lb_gb300")
        r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(root, "include"), p, "-L", lib, "-llbm_gb300",
                            "-Wl,-rpath," + lib, "-o", exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    f = np.ones((4, 5, 12), np.int32)
    f[:, :, 0] = 0
    f[:, :, 11] = 0
    f[:, 2, 6] = 0
    m = geometryMesherBoundary(dict(resolution_factor=1.0, additional_factor=0.5), {"flags": f})
    m.meshingBoundaryWall()
    m.meshingBoundaryConditionPeriodic(geometryObjectCuboid((0.9, -1, -1), (1.1, 99, 99), (1.0, 99, -1), -3),
                                       (-1, 0, 0), 10)
    m.meshingBoundaryConditionPeriodic(geometryObjectCuboid((9.9, -1, -1), (10.1, 99, 99), (10.0, -1, 99), -3),
                                       (1, 0, 0), 1)
    m.meshingBoundaryConditionInletUniform(geometryObjectCuboid((4.9, -1, -1), (5.1, 99, 99), (5.0, -1, 99), -1),
                                           (-1, 0, 0), (0.04, 0.0, 0.001))
    fo = fold_periodic(f, m.periodic, inlets=m.inlets)
    g = fo["flags"]
    s = int((g.reshape(-1).astype(np.int64) * np.arange(1, g.size + 1)).sum())
    want = [str(v) for v in (g.shape[2], g.shape[1], g.shape[0], *fo["periodic"], s, len(fo["inlets"]))]
    want += ["%d/%d/%d" % (r.vertex.x, r.vertex.y, r.vertex.z) for r in fo["inlets"]]
    assert out == want
    assert g.shape == (4, 5, 9) and (g == -1).sum() == 4 * 5
