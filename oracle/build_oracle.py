"""Build recipe for the CPU oracle (liboracle_mm3e.so).

TEST INFRASTRUCTURE ONLY: the oracle restates the MM3E CPU render path in C++ and is used as
the parity checker and as the timed CPU baseline. It is compiled without FP contraction
(`-ffp-contract=off`; GCC contracts by default on aarch64) because the reference is Rust,
which never fuses multiply-adds.

The reference itself (Rust, cargo) cannot be compiled on these machines, so there is no
`oracle/_ref` build; this restatement is the oracle.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle_mm3e.so")
SOURCES = ["oracle_capi.cpp"]
HEADERS = ["oracle_math.hpp", "oracle_count.hpp", "oracle_kit.hpp", "oracle_scene.hpp",
           os.path.join("..", "include", "mm3e_cuda.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = SOURCES + HEADERS + [os.path.basename(__file__)]
    return any(os.path.getmtime(os.path.join(HERE, d)) > t for d in deps)


def build(force=False, verbose=False):
    """Compile the oracle if any source is newer than the library. Returns the .so path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", "-Wall", "-Wno-unused-function", "-o", LIB + ".tmp"]
    cmd += [os.path.join(HERE, s) for s in SOURCES]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
