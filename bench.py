#!/usr/bin/env python
"""LJ atom-steps/s of the integer fixed-point MD step on GB300.

Workload (one step = one MD step of the whole system): 3D LJ liquid NVE, N = 1,048,576 atoms on
an FCC lattice at density 0.8442, Maxwell velocities at T = 0.72 (Threefry seed 1), cubic
periodic box, cutoff 2.5, Verlet skin 0.3 with displacement-triggered rebuilds, dt = 0.005,
integer fixed-point positions, f32 pair forces quantised to integer kicks. The state is
generated on the device and stays resident; the timed region replays the engine's captured
CUDA graphs (force + leapfrog every step, the list rebuild in a conditional node).

`--impl reference` times md-ref's CPU engine (restated in C++, IntEngine3<f32>'s reference loop,
all host threads) on the same workload.

One JSON line on stdout (rank 0). Multi-GPU (torchrun): one independent replica per GPU, barrier
+ max over ranks (replicas only: the path has no exchange step).
"""

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LJ atom-steps/s (plain vs batched/served, same GB300); p99 frame latency; FP64 err"
UNIT = "atom-steps/s"

N_ATOMS = 1 << 20
RHO, T0, SEED, SKIN, RC, DT = 0.8442, 0.72, 1, 0.3, 2.5, 0.005
# The slab workload states no skin: 0.4 ran fastest of 0.3, 0.4 and 0.5 on a GB300 (15.9e9 vs
# 15.1e9 and 15.8e9 atom-steps/s, frames excluded). The trajectory does not depend on the skin.
SKIN_SLAB = 0.4


def config_dict(extra=None):
    d = {
        "workload": f"3D LJ liquid NVE, FCC N={N_ATOMS}, rho 0.8442, T 0.72, rc 2.5, skin 0.3, dt 0.005 (plain form)",
        "n_atoms": N_ATOMS,
        "density": RHO,
        "temperature": T0,
        "cutoff": RC,
        "skin": SKIN,
        "dt": DT,
        "form": "plain (one system per launch sequence)",
        "l2": "inputs larger than L2 (neighbour list ~0.33 GB read per step, state 48 MB)",
    }
    if extra:
        d.update(extra)
    return d


def algorithmic_bytes_per_atom_step():
    """B = 2 S + 4 n_list: state read + written (S = 24 B positions + 12 B velocities) and one
    u32 index per listed neighbour, n_list = rho (4/3) pi (rc + skin)^3."""
    s = 24 + 12
    n_list = RHO * 4.0 / 3.0 * math.pi * (RC + SKIN) ** 3
    return 2 * s + 4 * n_list, n_list


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def profile_figure(key):
    """A figure of the committed ncu summary of the force kernel (`key: value` lines), if present."""
    path = os.path.join(ROOT, "profiles", "k_force_list_3d.md")
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1].split()[0])
    except Exception:
        pass
    return None


def profile_traffic():
    """DRAM bytes per force launch from the committed ncu summary, if present."""
    return profile_figure("dram_bytes_per_launch_full_size")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.file,
                stderr=subprocess.DEVNULL,
            )
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.flush()
        rows = []
        for line in open(self.file.name):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl"
        try:
            import torch

            if not torch.cuda.is_available():
                backend = "gloo"
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def barrier_max(pg, value):
    if pg is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def system3():
    from micrographia_gb300 import Pair, System3, cube_for

    return System3(cube_for(N_ATOMS, RHO), DT, Pair.lj(RC), [1.0])


def cpu_baseline(seconds_budget=20.0, threads=None, half3=True):
    """md-ref's CPU engine (C++ restatement of IntEngine3<f32>, OpenMP over all host threads) on the
    same workload; a bounded sample of steps. `half3`: its pair loop over half shells (each pair
    once, each side's kick rounded as the reference loop rounds it; the same kicks bit for bit,
    tests/test_oracle.py), else the reference loop itself."""
    from oracle import oracle as O

    threads = threads or os.cpu_count() or 1
    sys3 = system3()
    s0 = O.fcc_maxwell(sys3, N_ATOMS, T0, SEED, jitter=0.05)
    e = O.IntEngine(sys3, s0, threads=threads, half3=half3)
    e.step(5)  # warm-up: 5 steps, as the reference's own bench (crates/bench/src/main.rs:288)
    t0 = time.perf_counter()
    done = 0
    while done < 1 or (time.perf_counter() - t0 < seconds_budget and done < 64):
        e.step(1)
        done += 1
    dt = time.perf_counter() - t0
    # one thread, as the reference's own bench times its CPU engine (bench/src/main.rs:279-298)
    e1 = O.IntEngine(sys3, e.state, threads=1, half3=half3)
    t1 = time.perf_counter()
    e1.step(1)
    dt1 = time.perf_counter() - t1
    return {
        "value": N_ATOMS * done / dt,
        "unit": UNIT,
        "cores": threads,
        "kind": "port",
        "sample": f"{done} full steps of the {N_ATOMS}-atom system after 5 warm-up steps ({dt:.1f} s), IntEngine3<f32> "
        + ("over half shells (the reference loop's kicks bit for bit)" if half3 else "reference loop"),
        "single_thread": {"value": N_ATOMS / dt1, "unit": UNIT, "sample": f"1 full step on one thread ({dt1:.1f} s)"},
    }


def run_reference(args, world, rank, pg):
    if rank != 0:
        return 0
    # the reference's own algorithm: IntEngine3's loop over all 27 cells (it has no half-shell form)
    base = cpu_baseline(seconds_budget=min(60.0, 5.0 + 2.0 * args.steps), half3=False)
    line = {
        "metric": METRIC,
        "value": base["value"],
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": N_ATOMS / base["value"] * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+int64",
        "data": "synthetic",
        "impl": "reference",
        "config": config_dict(),
        "cpu_baseline": base,
        "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, world, rank, local, pg):
    import numpy as np
    import torch

    from micrographia_gb300 import ForceMode, GpuEngine3, _abi
    from micrographia_gb300.engine import make_init

    torch.cuda.set_device(local)
    sys3 = system3()
    spec = make_init(_abi.INIT_FCC, N_ATOMS, T0, SEED, 0.05)
    eng = GpuEngine3(sys3, None, ForceMode.verlet_with_skin(sys3, N_ATOMS, SKIN), init=spec, device=local)
    stream = torch.cuda.ExternalStream(eng.stream())

    # warm-up: captures the graphs and settles the lists
    eng.step(args.warmup)
    eng.wait()

    clocks = ClockSampler(local)
    clocks.start()
    l0 = eng.launch_count()
    if pg is not None:
        pg.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    eng.step(args.steps)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    eng.wait()
    clk = clocks.stop()
    launches = eng.launch_count() - l0
    ms = barrier_max(pg, ms)
    value = world * N_ATOMS * args.steps / (ms * 1e-3)
    rebuilds, overflow = eng.read_list_stats()

    # per-phase device times (CUDA events on the engine's stream) for the roofline
    lib = _abi.lib()
    import ctypes as C

    f_ms, r_ms, nreb = C.c_double(), C.c_double(), C.c_uint32()
    _abi.check(lib.gbmd_time_phases(eng._h, 200, C.byref(f_ms), C.byref(r_ms), C.byref(nreb)))
    B, n_list = algorithmic_bytes_per_atom_step()
    peaks, peak_kind = measured_peaks()
    achieved = B * N_ATOMS / (f_ms.value * 1e-3) / 1e9
    traffic = profile_traffic()

    # end to end through the public API with host buffers: upload from pinned host memory,
    # K steps, state read back to host memory
    st = eng.read_state()
    hp = torch.empty(st.pos.shape, dtype=torch.int64, pin_memory=True).numpy()
    hv = torch.empty(st.vel.shape, dtype=torch.int32, pin_memory=True).numpy()
    hs = torch.empty(st.species.shape, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    hp[:] = st.pos
    hv[:] = st.vel
    hs[:] = st.species
    from micrographia_gb300 import State3

    host_state = State3(hp, hv, hs)
    if pg is not None:
        pg.barrier()
    t0 = time.perf_counter()
    eng.upload(host_state)
    eng.step(args.steps)
    out = eng.read_state()
    t_e2e = barrier_max(pg, time.perf_counter() - t0)
    h2d = hp.nbytes + hv.nbytes + hs.nbytes
    d2h = out.pos.nbytes + out.vel.nbytes + out.species.nbytes
    e2e = {
        "value": world * N_ATOMS * args.steps / t_e2e,
        "unit": UNIT,
        "h2d_bytes_per_step": h2d / args.steps,
        "d2h_bytes_per_step": d2h / args.steps,
        "what": "gbmd_upload (pinned host state) + gbmd_step(K) + gbmd_read_state to host, per K steps",
    }

    # FP64 force error at full size (outside the timed regions): the f32 path's integer kicks
    # against the kicks of the same pair chain evaluated in f64 (IntEngine<f64>), relative RMS
    # as md-ref's physics test defines it (bar 1e-5)
    k32, _ = eng.kicks()
    k64, _ = eng.kicks_f64()
    d = k32.astype(np.float64) - k64.astype(np.float64)
    fp64_err = float(np.sqrt((d * d).sum() / (k64.astype(np.float64) ** 2).sum()))
    fp64_max = int(np.abs(d).max())

    # energy drift (outside the timed regions): total energy per atom every 100 steps over 4000
    # steps after 1000 more steps of equilibration, its least-squares slope per step and its range
    energy = energy_drift(eng, equilibrate=1000, steps=4000, every=100) if not args.no_drift else None

    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+int64",
        "data": "synthetic",
        "config": config_dict({"parallelism": f"replicas{world}" if world > 1 else "single"}),
        "e2e": e2e,
        "gpu_launches": launches,
        "roofline": {
            "bound": "hbm",
            "kernel": "k_force_list<3> (LJ force + leapfrog + trigger)",
            "achieved": achieved,
            "peak": peaks.get("hbm_gbs", 6800.0),
            "peak_kind": peak_kind,
            "unit": "GB/s",
            "frac": achieved / peaks.get("hbm_gbs", 6800.0),
            "traffic": traffic,
            "pipes_ncu_pct": {
                "issue_active": profile_figure("issue_active_pct"),
                "alu": profile_figure("alu_pipe_pct"),
                "fp32": profile_figure("fp32_pipe_pct"),
                "note": "the kernel is bound by the integer ALU pipe and instruction issue (profiles/k_force_list_3d.md)",
            },
            "algorithmic_bytes_per_atom_step": B,
            "n_list": n_list,
            "force_ms": f_ms.value,
        },
        "phases": {"force_ms": f_ms.value, "rebuild_ms": r_ms.value, "rebuilds_in_200": nreb.value, "rebuilds_timed_run": rebuilds},
        "energy": energy,
        "fp64_force_error": {"rel_rms": fp64_err, "max_abs_kick_diff": fp64_max, "bar": 1e-5, "n_atoms": N_ATOMS,
                             "reference": "kicks of the f64 pair chain (IntEngine<f64>) on the device, gbmd_kicks_f64"},
        "overflow": overflow,
    }
    if clk:
        line["clocks"] = clk
    eng.close()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    if not args.no_sub:
        # the batched and served forms against the plain form, on this GPU (whole job: every
        # rank runs them, units summed and times maxed over ranks)
        line["batched"] = run_c4(args, world, rank, local, pg, steps=100, warmup=5, emit=False)
        line["served"] = run_c5(args, world, rank, local, pg, requests=32, rate=64.0, emit=False)
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def energy_drift(eng, equilibrate, steps, every):
    """Total energy per atom (IntEngine's on-step kinetic energy + the pair potential, FP64) sampled
    every `every` steps over `steps` steps after `equilibrate` more: the least-squares slope per
    atom per step, the range, and the reference's bar for its 3D liquid (energy per particle within
    2e-3 over 5000 steps, crates/md/tests/three.rs:95-111)."""
    import numpy as np

    eng.step(equilibrate)
    ts, es = [], []
    for k in range(steps // every + 1):
        if k:
            eng.step(every)
        ke, pe = eng.energy()
        ts.append(k * every)
        es.append((ke + pe) / eng.n)
    t = np.array(ts, np.float64)
    e = np.array(es, np.float64)
    slope = float(np.polyfit(t, e, 1)[0])
    return {
        "e_per_atom_start": float(e[0]),
        "slope_per_atom_per_step": slope,
        "range_per_atom": float(e.max() - e.min()),
        "steps": steps,
        "after_equilibration_steps": equilibrate,
        "samples": len(es),
        "bar": "range per atom < 2e-3 over 5000 steps (crates/md/tests/three.rs:95-111)",
        "within_bar": bool(e.max() - e.min() < 2e-3),
    }


def run_c4(args, world, rank, local, pg, steps=None, warmup=None, emit=True):
    """1024 uneven 2D systems; batched (one persistent launch per step, 100-step
    graphs) against the plain form: one engine per system, run (a) one after another, each to the
    end of its steps before the next starts, and (b) all at once, each on its own stream. Every
    arm is warmed up with the same steps first, so that no graph is captured while timed."""
    import torch

    from micrographia_gb300 import BatchEngine, ForceMode, GpuEngine, init_state, workloads

    torch.cuda.set_device(local)
    K = steps or args.steps
    W = warmup or args.warmup
    cfg = workloads.config4(args.systems)
    systems = [s for s, _ in cfg]
    states = [init_state(s, sp.recipe, sp.n, sp.t, sp.seed, sp.jitter) for s, sp in cfg]
    total = sum(st.n() for st in states)
    mode = ForceMode.verlet_with_skin(None, 0, SKIN)

    # the autotuner times skins 0.3..0.7 sigma, then 2 and 4 force lanes per particle, on these
    # states (outside the timed region)
    batch = BatchEngine(systems, states, mode, block_steps=100, device=local, tune_skin=True)
    skin = batch.skin
    force_lanes = batch.force_lanes
    mode = ForceMode.verlet_with_skin(None, 0, skin)
    bstream = torch.cuda.ExternalStream(batch.stream())
    batch.step(W)
    batch.wait()
    clocks = ClockSampler(local)
    clocks.start()
    l0, r0 = batch.stats()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(bstream)
    batch.step(K)
    ev1.record(bstream)
    ev1.synchronize()
    ms_b = ev0.elapsed_time(ev1)
    batch.wait()
    clk = clocks.stop()
    l1, r1 = batch.stats()
    batch.step(2 * K)  # (untimed: to the plain arms' step count, for the identity check)
    batch.wait()
    from micrographia_gb300 import replicas

    # replicas: every rank runs the whole batch; units summed, time maxed over ranks
    units, secs = replicas.aggregate(pg, total * K, ms_b * 1e-3)
    value = units / secs
    plain = [GpuEngine(s, st, mode, device=local) for s, st in zip(systems, states)]
    for e in plain:
        e.step(W)
        e.step(K)  # warm-up: every graph the timed steps replay is captured here
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for e in plain:
        e.step(K)
    torch.cuda.synchronize()
    t_conc = time.perf_counter() - t0
    t0 = time.perf_counter()
    for e in plain:
        e.step(K)
        e.wait()
    t_serial = time.perf_counter() - t0
    value_conc = total * K / t_conc
    value_serial = total * K / t_serial
    checks = {}
    for k in (0, len(systems) - 1):
        checks[k] = plain[k].read_state() == batch.read_system(k)
    for e in plain:
        e.close()
    batch.close()
    rec = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": ms_b / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+int64",
        "data": "synthetic",
        "config": {
            "workload": f"{len(systems)} independent 2D LJ systems, N log-uniform [256, 65536] (sum {total}), rho U[0.3, 0.8], T U[0.5, 1.5], rc 2.5, dt 0.005",
            "skin": skin,
            "force_lanes": force_lanes,
            "skin_choice": "autotuned: fastest of 0.3..0.7 on two timed 100-step blocks per candidate, then of 1, 2 and 4 force lanes per particle at that skin; the plain forms use the same skin",
            "form": "batched: one persistent force launch per step over all systems, 100-step CUDA graphs",
            "plain_value": value_serial,
            "plain_form": "one engine per system, the systems run one after another (each synchronised before the next starts)",
            "batched_over_plain": value / value_serial,
            "plain_concurrent_value": value_conc,
            "plain_concurrent_form": "one engine per system, each stepped on its own stream, all issued back to back",
            "batched_over_plain_concurrent": value / value_conc,
            "replicas_bit_identical_to_plain": checks,
            "rebuilds": r1 - r0,
        },
        "gpu_launches": l1 - l0,
    }
    if clk:
        rec["clocks"] = clk
    if rank == 0 and emit:
        print(json.dumps(rec), flush=True)
    return rec


def run_c3(args, world, rank, local, pg):
    """2D liquid-vapour slab, N = 2^24, rescale to T = 0.45 every 10 steps, RDF (200
    bins to r = 5) and density profile (80 bins) every 100 steps inside the timed region."""
    import torch

    from micrographia_gb300 import ForceMode, GpuEngine, workloads

    torch.cuda.set_device(local)
    sys_, spec = workloads.config3(args.atoms if args.atoms != (1 << 20) else 1 << 24)
    n = spec.n
    eng = GpuEngine(sys_, None, ForceMode.verlet_with_skin(sys_, n, SKIN_SLAB), init=spec, rescale_every=10, rescale_t=0.45, device=local)
    stream = torch.cuda.ExternalStream(eng.stream())
    eng.step(args.warmup)
    eng.wait()
    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    done, frames = 0, []
    while done < args.steps:
        k = min(100, args.steps - done)
        eng.step(k)
        done += k
        if done % 100 == 0:
            f, rdf, prof = eng.observe(rdf_bins=200, rdf_rmax=5.0, profile_bins=80, profile_axis=0)
            frames.append({"step": done, "T": f.temperature, "P": f.pressure, "pe_per_atom": f.potential / n})
    ev1.record(stream)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    rebuilds, overflow = eng.read_list_stats()
    line = {
        "metric": METRIC,
        "value": world * n * args.steps / (wall),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": wall * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+int64",
        "data": "synthetic",
        "config": {
            "workload": f"2D liquid-vapour slab N={n}, 4:1 box, liquid 0.70 / vapour 0.05, rescale T=0.45 every 10 steps, RDF + profile every 100 steps, skin {SKIN_SLAB}",
            "timing": "wall clock including the frames (observables copied to the host every 100 steps)",
            "device_ms_last_event_pair": ms,
            "frames": frames[-3:],
            "rebuilds": rebuilds,
            "overflow": overflow,
        },
    }
    if clk:
        line["clocks"] = clk
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()
    return 0


def _pct(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = min(len(xs) - 1, max(0, int(math.ceil(q / 100.0 * len(xs))) - 1))
    return xs[k]


def run_c5(args, world, rank, local, pg, requests=None, rate=None, emit=True):
    """A Poisson stream of 2D/3D requests (N log-uniform in [1024, 2^20], 2000 steps,
    a frame of T, P and a 200-bin RDF every 100 steps) served under a 64 GB HBM budget, against
    the same requests run one after another in plain form. Per-frame latency: the wall time a
    client waits for each frame after the previous one of its request (after submission for the
    first)."""
    import torch

    from micrographia_gb300 import ForceMode, GpuEngine, GpuEngine3, Server, workloads

    from micrographia_gb300 import replicas

    torch.cuda.set_device(local)
    # replicas: the request stream is dealt out by rank (request k to rank k mod N)
    n_req = requests or args.requests
    lam = rate or args.rate
    reqs = replicas.shard(workloads.config5(n_req, lam), rank, world)
    steps = 2000

    # frame times per request (by its place in the stream): served deliveries, and the solo
    # schedule S_k = time from the start of service to frame k when the request runs alone
    served_at = [[] for _ in reqs]
    arrival = [t for t, _, _ in reqs]
    solo = [[] for _ in reqs]
    start_plain = [0.0] * len(reqs)

    lane_stats = {}

    def serve():
        frames_lat, done, t_arr, t_prev, order = [], 0, {}, {}, {}
        sv = Server(64 << 30, max_active=64, device=local, lane_max_n=0 if getattr(args, "no_lanes", False) else None)
        t0 = time.perf_counter()
        pending = list(enumerate(reqs))
        total = 0
        while done < len(reqs):
            now = time.perf_counter() - t0
            while pending and pending[0][1][0] <= now:
                idx, (_, s, spec) = pending.pop(0)
                rid = sv.submit(s, spec, steps=steps, frame_every=100, rdf_bins=200, rdf_rmax=5.0)
                t_arr[rid] = time.perf_counter() - t0
                t_prev[rid] = t_arr[rid]
                order[rid] = idx
                total += spec.n * steps
            got = sv.poll()
            tnow = time.perf_counter() - t0
            for f in got:
                frames_lat.append(tnow - t_prev[f.request])
                t_prev[f.request] = tnow
                served_at[order[f.request]].append(tnow)
                if f.last:
                    done += 1
            if not got:
                time.sleep(0.0002)
        makespan = time.perf_counter() - t0
        st = sv.stats()
        lane_stats.update(lane_requests=st.lane_requests, lane_repacks=st.lane_repacks)
        sv.close()
        return total / makespan, makespan, frames_lat

    def serial():
        frames_lat = []
        t0 = time.perf_counter()
        total = 0
        for idx, (t_a, s, spec) in enumerate(reqs):
            while time.perf_counter() - t0 < t_a:
                time.sleep(0.0005)
            t_prev = t0 + t_a  # the first frame's wait counts from the request's arrival
            t_start = time.perf_counter()
            start_plain[idx] = t_start - t0
            cls = GpuEngine if s.DIM == 2 else GpuEngine3
            e = cls(s, None, ForceMode.verlet_with_skin(s, spec.n, SKIN), init=spec, block_steps=100, device=local)
            for _ in range(0, steps, 100):
                e.step(100)
                e.observe(rdf_bins=200, rdf_rmax=5.0)
                t = time.perf_counter()
                frames_lat.append(t - t_prev)
                solo[idx].append(t - t_start)
                t_prev = t
            e.close()
            total += spec.n * steps
        makespan = time.perf_counter() - t0
        return total / makespan, makespan, frames_lat

    v_serve, mk_serve, lat_serve = serve()
    v_serial, mk_serial, lat_serial = serial()
    # lateness: delivery minus the frame's due time in the request's own schedule (arrival + S_k)
    late_serve = [served_at[q][k] - (arrival[q] + solo[q][k]) for q in range(len(reqs)) for k in range(min(len(served_at[q]), len(solo[q])))]
    late_serial = [start_plain[q] - arrival[q] for q in range(len(reqs)) for _ in solo[q]]
    late_serve = replicas.gather(pg, late_serve)
    late_serial = replicas.gather(pg, late_serial)
    # whole job over ranks: atom-steps summed, makespans maxed, latencies pooled
    u, mk_serve = replicas.aggregate(pg, v_serve * mk_serve, mk_serve)
    v_serve = u / mk_serve
    u, mk_serial = replicas.aggregate(pg, v_serial * mk_serial, mk_serial)
    v_serial = u / mk_serial
    lat_serve = replicas.gather(pg, lat_serve)
    lat_serial = replicas.gather(pg, lat_serial)
    line = {
        "metric": METRIC,
        "value": v_serve,
        "unit": UNIT,
        "n_gpus": world,
        "steps": steps,
        "warmup": args.warmup,
        "ms_per_step": None,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+int64",
        "data": "synthetic",
        "config": {
            "workload": f"{n_req} requests (dealt out over {world} GPU(s)), Poisson arrivals at {lam}/s, 50% 2D / 50% 3D LJ, N log-uniform [1024, 2^20], rho U[0.3, 0.85], T U[0.5, 1.5], {steps} steps, T/P/RDF frame every 100 steps, 64 GB HBM budget",
            "form": "served: continuous batching (requests of N <= 65,536 stepped together per dimension in a lane batch that they join and leave at frame boundaries, larger ones each on an engine of its own; all overlapped on the device)"
            if not getattr(args, "no_lanes", False)
            else "served: every request on an engine of its own, intervals overlapped",
            "lane_requests": lane_stats.get("lane_requests"),
            "lane_repacks": lane_stats.get("lane_repacks"),
            "makespan_s": mk_serve,
            "frame_latency_p50_ms": 1e3 * _pct(lat_serve, 50),
            "frame_latency_p99_ms": 1e3 * _pct(lat_serve, 99),
            "frame_lateness_p50_ms": 1e3 * _pct(late_serve, 50),
            "frame_lateness_p99_ms": 1e3 * _pct(late_serve, 99),
            "plain_frame_lateness_p50_ms": 1e3 * _pct(late_serial, 50),
            "plain_frame_lateness_p99_ms": 1e3 * _pct(late_serial, 99),
            "latency_definitions": "latency: wait for each frame after the previous one of its request (the first from arrival); lateness: delivery minus the frame's due time in the request's own schedule, arrival + the time the frame took from the start of service when the request ran alone (the plain arm's runs)",
            "plain_value": v_serial,
            "plain_makespan_s": mk_serial,
            "plain_frame_latency_p50_ms": 1e3 * _pct(lat_serial, 50),
            "plain_frame_latency_p99_ms": 1e3 * _pct(lat_serial, 99),
            "served_over_plain": v_serve / v_serial,
            "frames": len(lat_serve),
        },
    }
    if rank == 0 and emit:
        print(json.dumps(line), flush=True)
    return line


def main():
    global N_ATOMS
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=64)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sub", action="store_true", help="default line without the batched and served sub-records")
    ap.add_argument("--no-lanes", action="store_true", help="--config c5: serve every request on an engine of its own")
    ap.add_argument("--no-drift", action="store_true", help="default line without the energy-drift run")
    ap.add_argument("--atoms", type=int, default=N_ATOMS, help="atoms (default 1,048,576; smaller only for profiling)")
    ap.add_argument("--config", choices=["c2", "c3", "c4", "c5"], default="c2", help="c2 (default): 3D N=1M; c3: 2D slab 16.7M; c4: 1024 replicas; c5: served stream")
    ap.add_argument("--requests", type=int, default=48, help="requests for --config c5")
    ap.add_argument("--rate", type=float, default=8.0, help="Poisson arrival rate (1/s) for --config c5")
    ap.add_argument("--systems", type=int, default=1024, help="replicas for --config c4")
    args = ap.parse_args()
    N_ATOMS = args.atoms
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    world, rank, local, pg = dist_setup()
    if args.impl == "reference":
        rc = run_reference(args, world, rank, pg)
    else:
        from micrographia_gb300 import build

        build.build()
        if args.config == "c4":
            run_c4(args, world, rank, local, pg)
            rc = 0
        elif args.config == "c5":
            run_c5(args, world, rank, local, pg)
            rc = 0
        elif args.config == "c3":
            rc = run_c3(args, world, rank, local, pg)
        else:
            rc = run_ours(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
