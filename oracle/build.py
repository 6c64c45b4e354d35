"""Build recipe of the CPU oracle (test infrastructure): g++ on the two restatement files.

Output: oracle/_build/liboracle.so (git-ignored; rebuilt on every machine, x86 or Arm).
No -march=native: the same flags must work on the Arm GPU host.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "lbm_oracle.cpp"), os.path.join(HERE, "voxel_oracle.cpp")]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SOURCES + [os.path.join(HERE, "..", "include", "lbm.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    cmd = ["g++", "-O3", "-fopenmp", "-shared", "-fPIC", "-std=c++17", "-o", LIB + ".tmp"] + SOURCES
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
