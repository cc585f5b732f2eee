"""Build recipe of the engine: compiles the CUDA sources for sm_103a into the in-tree C-ABI
library micrographia_gb300/_build/libgbmd.so (no CPU fallback is built).

Every translation unit is compiled with -fmad=false so that no f32/f64 multiply-add is
contracted: the pair arithmetic must round exactly as the reference's unfused Rust floats do.
The units compile in parallel; the link is one nvcc -shared call.
"""

import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgbmd.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xcudafe", "--diag_suppress=177"]
UNITS = ["engine.cu", "sort.cu", "init.cu", "batch.cu", "noalloc.cu", "serve.cu", "selfcheck.cu"]


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "gbmd.h"), __file__]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps())


def _compile(unit, extra):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT, unit.replace(".cu", ".o"))
    cmd = ["nvcc", *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {unit}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force=False, verbose=False, extra=()):
    """Compile libgbmd.so if any source changed; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(lambda u: _compile(u, list(extra)), UNITS))
    if verbose:
        for _, err in results:
            if err.strip():
                print(err)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["nvcc", *ARCH, "-shared", "-o", tmp, *[o for o, _ in results], "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    print(build(force="--force" in sys.argv, verbose=v, extra=["-Xptxas", "-v"] if v else []))
