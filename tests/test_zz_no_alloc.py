"""lbm_voxelize_mesh_noalloc against lbm_voxelize_mesh, through the C ABI.

The allocation-free entry point serves callers that may not call cudaMalloc themselves (their
memory manager owns the device heap, or their loop must not allocate): they hand in a device
buffer for the flags and the library uses only a fixed array compiled into it.  Here the test
itself allocates that buffer (with torch, as such a caller's pool would), calls the entry point
twice in a row on two different meshes, larger first, and requires the flags to equal the
allocating voxelizer's bit for bit.  This file is collected last so that a failure here comes
after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from lb_gb300 import capi, cases

pytestmark = pytest.mark.gpu


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def reference_flags(v, t, res, add):
    L = capi.lib()
    dims = np.zeros(3, np.int32)
    bbox = np.zeros(6)
    assert L.lbm_voxelize_mesh(_dp(v), len(v), _ip(t), len(t), res, add, None, _ip(dims), _dp(bbox), 0) == 0
    out = np.zeros(int(dims.prod()), np.int32)
    assert L.lbm_voxelize_mesh(_dp(v), len(v), _ip(t), len(t), res, add, _ip(out), _ip(dims), _dp(bbox), 0) == 0
    return out, dims, bbox


def test_no_alloc_voxelizer_matches_allocating_entry_point(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = capi.lib()
    meshes = [
        (cases.perturbed_icosphere(radius=11.0, subdiv=3, lmax=6, amp=0.15), 1.0, 2.0),
        (cases.perturbed_icosphere(radius=6.0, subdiv=2, lmax=4, amp=0.10, seed=7), 1.5, 1.0),
    ]
    for (v, t), res, add in meshes:  # two calls in a row: the second must not see the first's state
        v = np.ascontiguousarray(v, dtype=np.float64)
        t = np.ascontiguousarray(t, dtype=np.int32)
        ref, rdims, rbbox = reference_flags(v, t, res, add)
        dims = np.zeros(3, np.int32)
        bbox = np.zeros(6)
        assert L.lbm_voxelize_mesh_noalloc(_dp(v), len(v), _ip(t), len(t), res, add, None, _ip(dims), _dp(bbox), 0) == 0
        assert np.array_equal(dims, rdims) and np.array_equal(bbox, rbbox)
        dev = torch.full((int(dims.prod()),), -7, dtype=torch.int32, device="cuda:0")
        rc = L.lbm_voxelize_mesh_noalloc(_dp(v), len(v), _ip(t), len(t), res, add, C.c_void_p(dev.data_ptr()),
                                         _ip(dims), _dp(bbox), 0)
        assert rc == 0
        got = dev.cpu().numpy()
        assert ref.sum() > 50
        assert np.array_equal(got, ref)


def test_no_alloc_voxelizer_rejects_oversized_input(built_lib):
    L = capi.lib()
    v = np.zeros((3, 3))
    v[1, 0] = 1.0
    v[2, 1] = 1.0
    t = np.zeros((40000, 3), np.int32)
    dims = np.zeros(3, np.int32)
    rc = L.lbm_voxelize_mesh_noalloc(_dp(v), 3, _ip(t), len(t), 1.0, 1.0, C.c_void_p(1), _ip(dims), None, 0)
    assert rc == capi.LBM_ERR_UNSUPPORTED


def test_no_alloc_voxelizer_rejects_a_bad_index_before_device_work(built_lib):
    """A triangle naming a vertex outside [0, nv) is rejected on the host, before any copy or kernel:
    the caller's device buffer keeps its contents."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = capi.lib()
    v, t = cases.perturbed_icosphere(radius=6.0, subdiv=2, lmax=4, amp=0.10, seed=7)
    v = np.ascontiguousarray(v, dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.int32)
    dims = np.zeros(3, np.int32)
    assert L.lbm_voxelize_mesh_noalloc(_dp(v), len(v), _ip(t), len(t), 1.0, 1.0, None, _ip(dims), None, 0) == 0
    t[len(t) // 2, 1] = len(v)
    dev = torch.full((int(dims.prod()),), -7, dtype=torch.int32, device="cuda:0")
    rc = L.lbm_voxelize_mesh_noalloc(_dp(v), len(v), _ip(t), len(t), 1.0, 1.0, C.c_void_p(dev.data_ptr()),
                                     _ip(dims), None, 0)
    assert rc == capi.LBM_ERR_INVALID
    assert bool((dev == -7).all())
