"""The legacy VTK writer and probe CSV (outputerVTK.h:26-851) on the CPU: the bytes of a small file equal
the layout restated independently here (float values, 6 significant digits, x fastest), and the
outputerVTK helpers name their fields as the reference does."""
import numpy as np

from lb_gb300 import output


def g6(v):
    return "%.6g" % float(np.float32(v))


def expected(title, dims, res, add, bbmin, fields):
    nx, ny, nz = dims
    N = nx * ny * nz
    r = np.float32(res)
    asp = g6(np.float32(1.0) / r)
    org = ["%.6g" % (float(np.float32(b)) - (float(np.float32(add)) - 0.5) / float(r)) for b in bbmin]
    s = ["# vtk DataFile Version 2.0", title, "ASCII", "DATASET STRUCTURED_POINTS",
         "DIMENSIONS %d %d %d" % dims, "ASPECT_RATIO %s %s %s" % (asp, asp, asp), "ORIGIN " + " ".join(org),
         "POINT_DATA %d" % N]
    for name, a, sc in fields:
        a = np.asarray(a, dtype=np.float64).reshape(-1)
        vals = (a.astype(np.float32) * np.float32(sc)).astype(np.float32)
        if a.size == N:
            s += ["SCALARS %s double 1" % name, "LOOKUP_TABLE default"] + [g6(v) for v in vals]
        else:
            v3 = vals.reshape(3, N)
            s += ["VECTORS %s double" % name] + [" ".join(g6(v3[c, q]) for c in range(3)) for q in range(N)]
    return "\n".join(s) + "\n"


def test_vtk_bytes_follow_the_reference_layout(built_lib, tmp_path):
    dims = (3, 2, 2)
    N = 12
    rng = np.random.default_rng(4)
    rho = 1.0 + 0.01 * rng.standard_normal(N)
    u = 0.05 * rng.standard_normal(3 * N)
    grid = output.Grid(dims, resolution=75.0, additional=3.0, bbmin=(-0.1, 0.0, 0.02))
    conv = {"Crho": 1.293, "Cpressure": 2.5e3, "Cu": 46.78}
    p = tmp_path / "variables.1.vtk"
    output.outputerVTK.variablesVTK(p, grid, rho, u, conv)
    want = expected("LBE variables", dims, 75.0, 3.0, (-0.1, 0.0, 0.02),
                    [("rho", rho, 1.293), ("p", rho / 3.0, 2.5e3), ("U", u, 46.78)])
    assert p.read_text() == want


def test_mesh_and_scalar_writers(built_lib, tmp_path):
    dims = (4, 3, 2)
    flags = np.array([0, 1, 10, -2] * 6, dtype=np.int32)
    grid = output.Grid(dims)
    p = tmp_path / "mesh.vtk"
    output.outputerVTK.MeshVTK(p, grid, flags, "BackwardStep")
    lines = p.read_text().splitlines()
    assert lines[1] == "LBE BackwardStep" and lines[8] == "SCALARS object double 1"
    assert lines[10:14] == ["0", "1", "10", "-2"] and len(lines) == 10 + 24
    f = np.arange(27 * 24, dtype=np.float64).reshape(27, 24) * 1e-3
    output.outputerVTK.distributionFunctionVTK(p, grid, f, 19)
    lines = p.read_text().splitlines()
    assert lines[8] == "SCALARS DFunciton_19 double 1" and lines[10] == g6(f[19, 0])
    output.outputerVTK.tauVTK(p, grid, np.full(24, 1.8))
    lines = p.read_text().splitlines()
    assert lines[8] == "SCALARS Tau double 1" and lines[10] == g6(np.float32(1) / np.float32(1.8))


def test_probe_csv_appends_rows(built_lib, tmp_path):
    p = tmp_path / "probeData.csv"
    conv = {"Crho": 1.293, "Cpressure": 2.5e3, "Cu": 46.78}
    output.outputerVTK.probeWriteOut(p, (0.01, -0.002, 0.0005, 1.001), conv, 1.25e-5)
    output.outputerVTK.probeWriteOut(p, (0.02, 0.0, 0.0, 0.999), conv, 1.25e-5)
    lines = p.read_text().splitlines()
    assert lines[0] == "Sampling frequency is: " + g6(1.25e-5) and lines[1] == "ux,uy,uz,rho,pressure"
    f = np.float32
    row = [f(f(0.01) * f(46.78)), f(f(-0.002) * f(46.78)), f(f(0.0005) * f(46.78)), f(f(1.001) * f(1.293)),
           f(f(f(1.001) * f(f(1.0) / f(3.0))) * f(2.5e3))]
    assert lines[2] == ",".join(g6(v) for v in row)
    assert len(lines) == 4


def test_restart_read_takes_the_lattice_dump_back(built_lib, tmp_path):
    """InitializationEquilibriumVariables.h:47-113: the first LOOKUP_TABLE block is rho and the
    "VECTORS U double" block u, each value read as a float.  A variablesLatticeVTK dump comes back as
    the float of its 6-digit text; a variablesVTK dump comes back scaled (the reference applies no
    conversion factor on this read)."""
    dims = (4, 3, 2)
    N = 24
    rng = np.random.default_rng(7)
    rho = 1.0 + 0.01 * rng.standard_normal(N)
    u = 0.05 * rng.standard_normal((3, N))
    grid = output.Grid(dims)
    p = tmp_path / "variables.vtk"
    output.outputerVTK.variablesLatticeVTK(p, grid, rho, u)
    r2, u2 = output.read_variables_vtk(p, dims)
    as_text = lambda a: np.array([float(np.float32(g6(v))) for v in np.asarray(a).reshape(-1)])
    assert np.array_equal(r2, as_text(rho)) and np.array_equal(u2.reshape(-1), as_text(u))
    assert np.abs(r2 - rho).max() < 1e-5 and np.abs(u2 - u).max() < 1e-6
    q = tmp_path / "physical.vtk"
    output.outputerVTK.variablesVTK(q, grid, rho, u, {"Crho": 2.0, "Cpressure": 1.0, "Cu": 10.0})
    r3, u3 = output.read_variables_vtk(q, dims)
    assert np.allclose(r3, 2.0 * rho, rtol=1e-5) and np.allclose(u3, 10.0 * u, rtol=1e-5, atol=1e-6)


def test_restart_read_rejects_bad_files(built_lib, tmp_path):
    import pytest
    from lb_gb300 import capi
    dims = (4, 3, 2)
    with pytest.raises(capi.LbmError) as e:
        output.read_variables_vtk(tmp_path / "missing.vtk", dims)
    assert e.value.status == capi.LBM_ERR_IO
    p = tmp_path / "v.vtk"
    output.outputerVTK.variablesLatticeVTK(p, output.Grid(dims), np.ones(24), np.zeros((3, 24)))
    with pytest.raises(capi.LbmError) as e:
        output.read_variables_vtk(p, (4, 3, 3))  # DIMENSIONS 4 3 2 in the file
    assert e.value.status == capi.LBM_ERR_INVALID
    text = p.read_text().splitlines()
    (tmp_path / "short.vtk").write_text("\n".join(text[:-3]) + "\n")
    with pytest.raises(capi.LbmError) as e:
        output.read_variables_vtk(tmp_path / "short.vtk", dims)
    assert e.value.status == capi.LBM_ERR_INVALID and "short velocity" in str(e.value)
    (tmp_path / "nou.vtk").write_text("\n".join(t for t in text if not t.startswith("VECTORS")) + "\n")
    with pytest.raises(capi.LbmError) as e:
        output.read_variables_vtk(tmp_path / "nou.vtk", dims)
    assert e.value.status == capi.LBM_ERR_INVALID


def test_cpp_outputers_write_the_python_files(built_lib, tmp_path):
    """outputerVTK / outputerMesh of the C++ mirror (include/lbm_solver.hpp): the same bytes as the Python
    writers for the same fields and constants, and MeshMatrixIn reads back what MeshMatrixOut wrote."""
    import os
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = tmp_path / "cpp"
    out.mkdir()
    src = r'''
#include <cstdio>
#include "lbm_solver.hpp"
using namespace lbm_gb300;
int main(int argc, char** argv) {
    LBMConstants C; LBMData D;
    C.dimX_int = 3; C.dimY_int = 2; C.dimZ_int = 2; C.results_dir = argv[1];
    C.resolution_factor = 75.0; C.additional_factor = 3.0; C.BBmin[0] = -0.1; C.BBmin[2] = 0.02;
    C.BBmax[0] = 0.2; C.BBmax[1] = 0.05; C.BBmax[2] = 0.09;
    C.Crho = 1.293; C.Cpressure = 2.5e3; C.Cu = 46.78; C.Ct = 1e-4; C.probe_every_it = 5;
    for (int q = 0; q < 12; q++) {
        D.rho.push_back(1.0 + 0.001 * q);
        D.meshFluid.push_back(q % 3 == 0 ? 0 : (q % 5 == 0 ? -1 : 1 + q));
    }
    for (int q = 0; q < 36; q++) D.u.push_back(0.01 * (q - 17));
    D.rhoTimeAvg = D.rho; D.uTimeAvg = D.u;
    for (int q = 0; q < 27 * 12; q++) D.df.push_back(0.001 * q - 0.1);
    outputerVTK::distributionFunctionVTK(D, C, 13, false);
    outputerVTK::variablesVTK(D, C, 4, false);
    outputerVTK::variablesLatticeVTK(D, C, 4, false);
    outputerVTK::variablesTimeAvgVTK(D, C, false);
    outputerVTK::MeshVTK(D, C, "meshIN");
    outputerVTK::probeWriteOut(C, 0.01, -0.02, 0.003, 1.001);
    outputerMesh::MeshMatrixOut(D, C, "geom");
    LBMConstants C2; LBMData D2; C2.results_dir = argv[1];
    outputerMesh::MeshMatrixIn(D2, C2, "geom", false);
    std::printf("%d %d %d %d\n", (int)(D2.meshFluid == D.meshFluid), C2.dimX_int, C2.dimY_int, C2.dimZ_int);
    return 0;
}
'''
    p = tmp_path / "t.cpp"
    exe = tmp_path / "t"
    p.write_text(src)
    lib = os.path.join(root, "lb_gb300")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(root, "include"), str(p), "-L", lib,
                        "-llbm_gb300", "-Wl,-rpath," + lib, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    res = subprocess.run([str(exe), str(out)], capture_output=True, text=True, check=True).stdout.split()
    assert res == ["1", "3", "2", "2"]
    N = 12
    rho = 1.0 + 0.001 * np.arange(N)
    u = 0.01 * (np.arange(3 * N) - 17)
    flags = np.array([0 if q % 3 == 0 else (-1 if q % 5 == 0 else 1 + q) for q in range(N)])
    grid = output.Grid((3, 2, 2), resolution=75.0, additional=3.0, bbmin=(-0.1, 0.0, 0.02))
    conv = {"Crho": 1.293, "Cpressure": 2.5e3, "Cu": 46.78}
    py = tmp_path / "py"
    py.mkdir()
    output.outputerVTK.variablesVTK(py / "variables.4.vtk", grid, rho, u, conv)
    output.outputerVTK.variablesLatticeVTK(py / "variablesLattice4.vtk", grid, rho, u)
    output.outputerVTK.variablesTimeAvgVTK(py / "variablesTimeAvg.vtk", grid, rho, u, conv)
    output.outputerVTK.MeshVTK(py / "meshIN.vtk", grid, flags, "meshIN")
    output.outputerVTK.distributionFunctionVTK(py / "distributionFunction13.vtk", grid,
                                               0.001 * np.arange(27 * N) - 0.1, 13)
    output.outputerVTK.probeWriteOut(py / "probeData.csv", [0.01, -0.02, 0.003, 1.001], conv, 1e-4 * 5)
    for name in ("variables.4.vtk", "variablesLattice4.vtk", "variablesTimeAvg.vtk", "meshIN.vtk", "probeData.csv",
                 "distributionFunction13.vtk"):
        assert (out / name).read_bytes() == (py / name).read_bytes(), name
