"""Build liblbm_gb300.so in-tree with nvcc for sm_103a (one -gencode, translation units in parallel).

Output: lb_gb300/liblbm_gb300.so (git-ignored), objects in lb_gb300/_build/.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblbm_gb300.so")
DRIVER = os.path.join(HERE, "lbm_run")          # C++ host driver (lb_gb300/host/lbm_run.cpp)
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]
# extra nvcc flags for tuning experiments (e.g. LBM_NVCC_EXTRA="-DLBM_STEP2_MIN_BLOCKS=5")
NVCC_FLAGS += os.environ.get("LBM_NVCC_EXTRA", "").split()
STEP_UNITS = [f"lbm_step_{s}_{c}.cu" for s in ("f16", "f32", "f64") for c in ("srt", "cum15", "cum17", "comb")]
UNITS = STEP_UNITS + ["lbm_step_f64.cu", "lbm_step_f32.cu", "lbm_step_f16.cu", "lbm_capi.cu", "voxelizer.cu", "mlp.cu",
                      "mesh_io.cu", "mesher.cu", "vtk_io.cu", "config_io.cu"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _deps_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "lbm.h"), __file__]
    return max(os.path.getmtime(f) for f in files)


def build_driver(force=False):
    """g++ the C++ host driver against the library (rpath next to it)."""
    src = os.path.join(HERE, "host", "lbm_run.cpp")
    deps = [src, os.path.join(INCLUDE, "lbm.h"), os.path.join(INCLUDE, "lbm_solver.hpp"), LIB]
    if not force and os.path.exists(DRIVER) and os.path.getmtime(DRIVER) >= max(os.path.getmtime(f) for f in deps):
        return DRIVER
    gxx = shutil.which("g++") or "g++"
    cmd = [gxx, "-O2", "-std=c++17", "-Wall", "-I", INCLUDE, src, "-L", HERE, "-llbm_gb300",
           "-Wl,-rpath,$ORIGIN", "-o", DRIVER + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed on lbm_run.cpp:\n{r.stderr}")
    os.replace(DRIVER + ".tmp", DRIVER)
    return DRIVER


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        build_driver()
        return LIB
    exe = nvcc()

    def compile_one(unit):
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        cmd = [exe] + NVCC_FLAGS + ["-c", os.path.join(CSRC, unit), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {unit}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(len(UNITS), max(4, os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, UNITS))
    tmp = LIB + ".tmp"
    cmd = [exe] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    build_driver(force=True)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
