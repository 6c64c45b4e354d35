"""Generate the voxelizer golden fixture from the reference's committed files.

Reads (in the reference checkout, read-only):
  3D/preprocess/BackwardStepLaminar.off          - input NOFF mesh (12 vertices, 20 triangles)
  3D/simulation/results/BackwardStepLaminar.txt  - the reference voxelizer's output matrix
and writes, next to this script:
  BackwardStepLaminar.off                        - the input mesh, byte-for-byte
  backward_step_laminar.npz                      - dims, header values and the 0/1 matrix,
                                                   bit-packed (x fastest, then y, then z), and the
                                                   SHA-256 of the matrix text file

The mesh-matrix text format is the reference's outputerMesh::MeshMatrixOut
(3D/preprocess/src/postprocesors/outputerMesh.h:19-56): a 9-line header, then the values
with x fastest, one row per (y, z) and a blank line after every z slice.
Run:  python tests/golden/make_golden.py <reference_root>   (the reference checkout's top directory)
"""
import hashlib
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_mesh_matrix(path):
    header = {}
    vals = []
    with open(path) as fh:
        for line in fh:
            if ":" in line:
                key, rest = line.split(":", 1)
                header[key.strip()] = rest.split()
                continue
            if line.strip():
                vals.extend(int(t) for t in line.split())
    nx, ny, nz = (int(t) for t in header["Dimensions"])
    arr = np.asarray(vals, dtype=np.int32)
    assert arr.size == nx * ny * nz, (arr.size, nx, ny, nz)
    return header, (nx, ny, nz), arr


def main(ref_root):
    off = os.path.join(ref_root, "3D/preprocess/BackwardStepLaminar.off")
    txt = os.path.join(ref_root, "3D/simulation/results/BackwardStepLaminar.txt")
    header, dims, arr = parse_mesh_matrix(txt)
    assert set(np.unique(arr).tolist()) <= {0, 1}
    shutil.copyfile(off, os.path.join(HERE, "BackwardStepLaminar.off"))
    np.savez_compressed(
        os.path.join(HERE, "backward_step_laminar.npz"),
        dims=np.asarray(dims, dtype=np.int32),
        resolution=np.float64(header["Resolution Factor"][0]),
        additional=np.float64(header["Additional Factor"][0]),
        bbmin=np.asarray([float(header[k][0]) for k in ("BBminx", "BBminy", "BBminz")]),
        bbmax=np.asarray([float(header[k][0]) for k in ("BBmaxx", "BBmaxy", "BBmaxz")]),
        packed=np.packbits(arr.astype(np.uint8)),
        count_inside=np.int64(arr.sum()),
        # SHA-256 of the reference's matrix file: the mesh-matrix writer must reproduce it byte for byte
        txt_sha256=np.array(hashlib.sha256(open(txt, "rb").read()).hexdigest()),
    )
    print("dims", dims, "inside", int(arr.sum()), "of", arr.size)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference_root>")
    main(sys.argv[1])
