"""Build recipe of the oracle (test infrastructure only).

Compiles the C++17 restatement of micrographia's CPU engine (oracle.hpp, capi.cpp) into
oracle/_build/liboracle.so. The flags keep the Rust floating-point semantics the oracle restates:
no contraction into fused multiply-adds, no fast-math. OpenMP parallelises the reference loop for
the multi-core CPU baseline. Host-portable: the same flags build on x86-64 and aarch64.
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "capi.cpp")]
HEADERS = [os.path.join(HERE, h) for h in ("oracle.hpp", "fdlibm.hpp")] + [
    os.path.join(HERE, "..", "include", "gbmd.h")
]
FLAGS = ["-std=c++17", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unknown-pragmas"]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in SOURCES + HEADERS)


def build(force: bool = False) -> str:
    """Compile liboracle.so if needed and return its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["g++", *FLAGS, "-o", tmp, *SOURCES]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
