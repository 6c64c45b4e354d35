"""The reference's mesh-matrix text files (postprocesors/outputerMesh.h:19-211) through the C ABI, on
the host: the writer reproduces the reference's committed matrix file byte for byte (its SHA-256 is
in the golden fixture), and the reader returns what the writer wrote."""
import ctypes as C
import hashlib
import os

import numpy as np
import pytest

from lb_gb300 import capi, cases

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "backward_step_laminar.npz")


def test_writer_reproduces_the_reference_file(built_lib, tmp_path):
    d = np.load(GOLD)
    nx, ny, nz = (int(v) for v in d["dims"])
    flags = np.unpackbits(d["packed"])[:nx * ny * nz].astype(np.int32).reshape(nz, ny, nx)
    p = str(tmp_path / "BackwardStepLaminar.txt")
    cases.write_mesh_matrix(p, flags, float(d["resolution"]), float(d["additional"]),
                            np.concatenate([d["bbmin"], d["bbmax"]]))
    with open(p, "rb") as fh:
        assert hashlib.sha256(fh.read()).hexdigest() == str(d["txt_sha256"])


def test_round_trip_with_boundary_flags(built_lib, tmp_path):
    rng = np.random.default_rng(3)
    flags = rng.integers(-3, 28, size=(5, 7, 9)).astype(np.int32)
    p = str(tmp_path / "m.txt")
    bbox = (-1.25, 0.5, 2.0, 10.0, 20.5, 30.125)
    cases.write_mesh_matrix(p, flags, 0.1, 2.0, bbox)
    f, r, a, bb = cases.read_mesh_matrix(p)
    assert np.array_equal(f, flags)
    assert abs(r - 0.1) < 1e-6 and a == 2.0 and np.allclose(bb, bbox)


def test_reader_errors(built_lib, tmp_path):
    L = capi.lib()
    dims = np.zeros(3, np.int32)
    ip = dims.ctypes.data_as(C.POINTER(C.c_int32))
    assert L.lbm_mesh_matrix_read(str(tmp_path / "missing.txt").encode(), None, 0, ip, None, None, None) == \
        capi.LBM_ERR_IO
    p = str(tmp_path / "m.txt")
    cases.write_mesh_matrix(p, np.ones((2, 3, 4), np.int32), 1.0, 1.0, (0, 0, 0, 1, 1, 1))
    small = np.zeros(5, np.int32)
    assert L.lbm_mesh_matrix_read(p.encode(), small.ctypes.data_as(C.POINTER(C.c_int32)), 5, ip, None, None,
                                  None) == capi.LBM_ERR_INVALID
    with pytest.raises(capi.LbmError):
        with open(p, "w") as fh:
            fh.write("not a mesh matrix\n")
        cases.read_mesh_matrix(p)
