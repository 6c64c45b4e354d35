"""Build recipe of the CPU oracle (test infrastructure): g++ on the two restatement files.

Output: oracle/_build/liboracle.so (git-ignored; rebuilt on every machine, x86 or Arm): portable flags,
the library the parity tests load.  build(native=True) makes oracle/_build/liboracle_native.so for the
timed CPU baseline only: the same sources tuned for the host's own cores (-mcpu=native on Arm,
-march=native on x86), with -ffp-contract=off as in the portable build (GCC would otherwise fuse
products into FMAs), so both libraries compute the same numbers.
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "lbm_oracle.cpp"), os.path.join(HERE, "voxel_oracle.cpp")]


BASE_FLAGS = ["-O3", "-fopenmp", "-shared", "-fPIC", "-std=c++17", "-ffp-contract=off"]


def native_flags():
    """Host-tuned code generation for the timed baseline: -mcpu=native on Arm, -march=native on x86."""
    return ["-mcpu=native"] if platform.machine().lower() in ("aarch64", "arm64") else ["-march=native"]


def build(force=False, native=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    lib = os.path.join(OUT_DIR, "liboracle_native.so") if native else LIB
    newest = max(os.path.getmtime(s) for s in SOURCES + [os.path.join(HERE, "..", "include", "lbm.h"), __file__])
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= newest:
        return lib
    cmd = ["g++"] + BASE_FLAGS + (native_flags() if native else []) + ["-o", lib + ".tmp"] + SOURCES
    subprocess.run(cmd, check=True)
    os.replace(lib + ".tmp", lib)
    return lib


def flags(native=False):
    return " ".join(["g++"] + BASE_FLAGS + (native_flags() if native else []))


if __name__ == "__main__":
    print(build(force=True))
