"""Race freedom of the in-place AA streaming, by emulating on the CPU the element addresses the packed-pair
step kernels touch (load_pair / store_pair with the periodic-x seam indices eL, eR, and load_pair_rows /
store_pair_rows on periodic y/z seams, lbm_step.cuh; the per-direction base addresses of make_params,
lbm_capi.cu).  For every pair thread of small fully periodic lattices, on even and odd steps:
  * direction v reads slot v of its own cells (even) or slot opp(v) of cell x - c_v (odd), and writes
    slot opp(v) of its own cells (even) or slot v of x + c_v (odd), with periodic wrap: the AA pattern;
  * the elements a thread writes are exactly the elements it read, so no other thread touches them;
  * the threads' element sets partition the 27 N elements of the population array.
The same for the row-staged kernel's shared segments, halo fill and fold (lbm_tma.cuh).  The velocity
table is read from the kernels' own source."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def velocity_table():
    src = open(os.path.join(ROOT, "lb_gb300", "csrc", "lbm_math.cuh")).read()
    out = []
    for name in ("cx", "cy", "cz"):
        m = re.search(r"constexpr int %s\(int v\) \{\s*constexpr int t\[27\] = \{([^}]*)\}" % name, src)
        out.append([int(t) for t in m.group(1).split(",")])
    return np.array(out).T  # [27, 3]


CV = velocity_table()


def opp(v):
    return 0 if v == 0 else (v + 1 if v & 1 else v - 1)


def pair_elements(nx, ny, nz, x0, y, z, odd):
    """(reads, writes): per direction v the two (slot, element) pairs the pair thread (x0, x0+1, y, z) loads
    and stores, following the kernels' index arithmetic."""
    N, nxy = nx * ny * nz, nx * ny
    idx0 = (z * ny + y) * nx + x0
    yz_seam = y in (0, ny - 1) or z in (0, nz - 1)  # every axis wraps here
    reads, writes = {}, {}
    if not yz_seam:
        e0, e1 = idx0, idx0 + 1
        eL = e0 + nx if x0 == 0 else e0
        eR = e1 - nx if x0 + 2 == nx else e1
        for v in range(27):
            cx, cy, cz = CV[v]
            off = cx + cy * nx + cz * nxy
            if not odd:
                rb, wb = v * N, opp(v) * N
                reads[v] = [rb + e0, rb + e0 + 1]
                writes[v] = [wb + e0, wb + e0 + 1]
                continue
            rb, wb = opp(v) * N - off, v * N + off
            if cx > 0:
                reads[v] = [rb + eL, rb + e1]
                writes[v] = [wb + e0, wb + eR]
            elif cx < 0:
                reads[v] = [rb + e0, rb + eR]
                writes[v] = [wb + eL, wb + e1]
            else:
                reads[v] = [rb + e0, rb + e0 + 1]
                writes[v] = [wb + e0, wb + e0 + 1]
    else:
        R = {}
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                R[(dy, dz)] = (((z + dz) % nz) * ny + (y + dy) % ny) * nx
        xm = nx - 1 if x0 == 0 else x0 - 1
        x2 = 0 if x0 + 2 == nx else x0 + 2
        for v in range(27):
            cx, cy, cz = CV[v]
            rslot, wslot = (opp(v), v) if odd else (v, opp(v))
            rrow = R[(-cy, -cz)] if odd else R[(0, 0)]
            wrow = R[(cy, cz)] if odd else R[(0, 0)]
            if odd and cx > 0:
                ri, wi = (xm, x0), (x0 + 1, x2)
            elif odd and cx < 0:
                ri, wi = (x0 + 1, x2), (xm, x0)
            else:
                ri = wi = (x0, x0 + 1)
            reads[v] = [rslot * N + rrow + i for i in ri]
            writes[v] = [wslot * N + wrow + i for i in wi]
    return reads, writes


def aa_expected(nx, ny, nz, x, y, z, v, odd):
    """The AA pattern: the element direction v reads and the one it writes for cell (x, y, z)."""
    N = nx * ny * nz

    def cell(a, b, c):
        return ((c % nz) * ny + b % ny) * nx + a % nx

    cx, cy, cz = CV[v]
    if not odd:
        return v * N + cell(x, y, z), opp(v) * N + cell(x, y, z)
    return opp(v) * N + cell(x - cx, y - cy, z - cz), v * N + cell(x + cx, y + cy, z + cz)


@pytest.mark.parametrize("shape", [(4, 3, 3), (6, 4, 5), (8, 5, 3), (2, 3, 4)])
@pytest.mark.parametrize("odd", [False, True])
def test_pair_threads_follow_aa_and_partition_the_array(shape, odd):
    nx, ny, nz = shape
    N = nx * ny * nz
    owner = np.full(27 * N, -1, np.int64)
    for z in range(nz):
        for y in range(ny):
            for x0 in range(0, nx, 2):
                reads, writes = pair_elements(nx, ny, nz, x0, y, z, odd)
                for v in range(27):
                    for lane in range(2):
                        r, w = aa_expected(nx, ny, nz, x0 + lane, y, z, v, odd)
                        assert reads[v][lane] == r and writes[v][lane] == w, (x0, y, z, v, lane)
                rs = sorted(e for v in range(27) for e in reads[v])
                ws = sorted(e for v in range(27) for e in writes[v])
                assert rs == ws and len(set(ws)) == 54
                tid = (z * ny + y) * nx + x0
                assert (owner[ws] == -1).all()
                owner[ws] = tid
    assert (owner >= 0).all()


def row_segment(nx, ny, nz, V, y, z, odd):
    """Global element index of position 0 of segment V of row (y, z) (row_segment, lbm_tma.cuh)."""
    N = nx * ny * nz
    slot, yy, zz = V, y, z
    if odd:
        slot = opp(V)
        yy = (y - CV[V][1]) % ny
        zz = (z - CV[V][2]) % nz
    return slot * N + (zz * ny + yy) * nx


@pytest.mark.parametrize("shape", [(6, 3, 4), (8, 4, 3)])
@pytest.mark.parametrize("odd", [False, True])
def test_row_staged_segments_follow_aa(shape, odd):
    """The row-staged kernel (lbm_tma.cuh row_from_stage): through its shared segments, periodic halo fill
    and fold, every cell reads the AA element of each direction and every stored position receives the
    post-collision value the AA pattern puts there; the 27 segments of a row are read and written back
    whole, and the rows' segments partition the array."""
    nx, ny, nz = shape
    N = nx * ny * nz
    owner = np.full(27 * N, -1, np.int64)
    for z in range(nz):
        for y in range(ny):
            base = [row_segment(nx, ny, nz, V, y, z, odd) for V in range(27)]
            for V in range(27):
                seg = np.arange(base[V], base[V] + nx)
                assert (owner[seg] == -1).all()
                owner[seg] = z * ny + y
            # stage[V][1 + pos], pos in [-1, nx]: element ids fetched (halo positions empty)
            stage = [[None] + [base[V] + x for x in range(nx)] + [None] for V in range(27)]
            if odd:  # halo fill
                for V in range(27):
                    if CV[V][0] > 0:
                        stage[V][0] = stage[V][nx]
                    elif CV[V][0] < 0:
                        stage[V][nx + 1] = stage[V][1]
            for x in range(nx):
                for V in range(27):
                    sh = -CV[V][0] if odd else 0
                    r, _ = aa_expected(nx, ny, nz, x, y, z, V, odd)
                    assert stage[V][1 + x + sh] == r, (x, y, z, V)
            out = [[None] * (nx + 2) for _ in range(27)]
            for x in range(nx):
                for V in range(27):
                    sh = CV[V][0] if odd else 0
                    out[opp(V)][1 + x + sh] = (x, V)
            if odd:  # halo fold
                for V in range(27):
                    if CV[V][0] < 0:
                        out[V][1] = out[V][nx + 1]
                    elif CV[V][0] > 0:
                        out[V][nx] = out[V][0]
            for V in range(27):
                for x in range(nx):
                    cell_x, v = out[V][1 + x]
                    _, w = aa_expected(nx, ny, nz, cell_x, y, z, v, odd)
                    assert w == base[V] + x, (x, y, z, V)
    assert (owner >= 0).all()
