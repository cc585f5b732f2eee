"""Bench results as JSON lines in the schema of micrographia's bench/results.jsonl
(crates/bench/src/main.rs:262-277): time, commit, device, engine, mode, order, dim, pair,
density, n, steps_per_s, ns_per_particle_step, phase_ns, copy_gbps; followed, when known, by this
engine's own figures (atom_steps_per_s, roofline_fraction, force_err_rms, energy_drift_per_step,
p50_ms, p99_ms), so the numbers can be tracked beside the reference's history.

    python -m micrographia_gb300.results --dim 3 --sizes 32000,262144,1048576 --density 0.8442 \\
        --save results.jsonl

measures each size on the GPU (a fluid on a lattice, Verlet lists, 'lj' or 'wca') and appends
one line per size."""

import argparse
import json
import os
import subprocess
import time

KEYS = ("time", "commit", "device", "engine", "mode", "order", "dim", "pair", "density", "n", "steps_per_s",
        "ns_per_particle_step", "phase_ns", "copy_gbps")
EXTRA = ("atom_steps_per_s", "roofline_fraction", "force_err_rms", "energy_drift_per_step", "p50_ms", "p99_ms")


def record(*, engine, mode, order, dim, pair, density, n, steps_per_s, phase_ns, copy_gbps, commit="", device="", when=None,
           **extra):
    """One result line as an ordered dict: the reference's fields, then the extra figures given."""
    unknown = set(extra) - set(EXTRA)
    if unknown:
        raise ValueError(f"unknown result fields {sorted(unknown)}")
    rec = {
        "time": int(when if when is not None else time.time()),
        "commit": commit,
        "device": device,
        "engine": engine,
        "mode": mode,
        "order": order,
        "dim": int(dim),
        "pair": pair,
        "density": float(density),
        "n": int(n),
        "steps_per_s": round(float(steps_per_s), 1),
        "ns_per_particle_step": round(1e9 / (float(steps_per_s) * int(n)), 3),
        "phase_ns": {k: int(round(v)) for k, v in phase_ns.items()},
        "copy_gbps": round(float(copy_gbps), 1),
    }
    for k in EXTRA:
        if k in extra and extra[k] is not None:
            rec[k] = extra[k]
    return rec


def dumps(rec):
    return json.dumps(rec, separators=(",", ":"))


def append(path, records):
    with open(path, "a") as f:
        for r in records:
            f.write(dumps(r) + "\n")


def _commit():
    try:
        return subprocess.run(["git", "rev-parse", "--short", "HEAD"], capture_output=True, text=True, timeout=10,
                              cwd=os.path.dirname(os.path.abspath(__file__))).stdout.strip()
    except Exception:
        return ""


def copy_gbps(device=0, mib=1024):
    """Device copy bandwidth (read + write), as the reference's bench reports it."""
    import torch

    a = torch.empty(mib << 20, dtype=torch.uint8, device=f"cuda:{device}")
    b = torch.empty_like(a)
    for _ in range(3):
        b.copy_(a)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        b.copy_(a)
    e1.record()
    e1.synchronize()
    return 2 * 10 * a.numel() / (e0.elapsed_time(e1) * 1e-3) / 1e9


def measure(dim, n, density, pair="lj", steps=1000, skin=0.3, arith=0, device=0, copy=None):
    """One case on the GPU: a seeded fluid (2D lattice + jitter, 3D FCC) at T = 1 (0.72 in 3D),
    Verlet lists; steps/s over `steps` steps, phase times from gbmd_time_phases."""
    import ctypes as C

    import torch

    from . import _abi
    from .core import Pair, System, System3, box_for, cube_for
    from .engine import ForceMode, GpuEngine, GpuEngine3, make_init

    p = Pair.lj(2.5) if pair == "lj" else Pair.wca()
    if dim == 2:
        sys_ = System(box_for(n, density, 1.0), 0.005, p, [1.0])
        spec = make_init(_abi.INIT_FLUID, n, 1.0, 1, 0.1)
        eng = GpuEngine(sys_, None, ForceMode.verlet_with_skin(sys_, n, skin), init=spec, device=device, arith=arith)
    else:
        sys_ = System3(cube_for(n, density), 0.005, p, [1.0])
        spec = make_init(_abi.INIT_FCC, n, 0.72, 1, 0.05)
        eng = GpuEngine3(sys_, None, ForceMode.verlet_with_skin(sys_, n, skin), init=spec, device=device, arith=arith)
    with eng:
        eng.step(64)
        eng.wait()
        st = torch.cuda.ExternalStream(eng.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        eng.step(steps)
        e1.record(st)
        e1.synchronize()
        sps = steps / (e0.elapsed_time(e1) * 1e-3)
        f, r, nr = C.c_double(), C.c_double(), C.c_uint32()
        _abi.check(_abi.lib().gbmd_time_phases(eng._h, 200, C.byref(f), C.byref(r), C.byref(nr)))
    phases = {"force": f.value * 1e6, "rebuild": r.value * 1e6 * nr.value / 200.0}
    return record(engine="gb300-int-int" if arith else "gb300-int-f32", mode="verlet", order="lattice", dim=dim, pair=pair,
                  density=density, n=n, steps_per_s=sps, phase_ns=phases,
                  copy_gbps=copy if copy is not None else copy_gbps(device), commit=_commit(),
                  device=torch.cuda.get_device_name(device) + " (CUDA)", atom_steps_per_s=sps * n)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--dim", type=int, default=3, choices=[2, 3])
    ap.add_argument("--sizes", default="32000,262144,1048576")
    ap.add_argument("--density", type=float, default=0.8442)
    ap.add_argument("--pair", default="lj", choices=["lj", "wca"])
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--int", action="store_true", help="all-integer table forces")
    ap.add_argument("--save", default=None, help="append the lines to this file")
    a = ap.parse_args(argv)
    bw = copy_gbps()
    recs = [measure(a.dim, int(s), a.density, a.pair, a.steps, arith=1 if a.int else 0, copy=bw) for s in a.sizes.split(",")]
    for r in recs:
        print(dumps(r))
    if a.save:
        append(a.save, recs)


if __name__ == "__main__":
    main()
