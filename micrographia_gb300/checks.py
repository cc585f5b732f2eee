"""Engine self-checks (crates/md/src/checks.rs): the same names and scenarios, run on the GPU.

`run(name)` returns (ok, message) where the reference returns Ok(message) / Err(message). Every
check runs on this package's engines alone: initial conditions come from the device initialiser,
and `md_kicks_vs_cpu`, whose reference takes its state from 100 steps of the CPU twin and
compares kicks with IntEngine<f64>'s, steps the GPU engine instead (the same bits) and compares
with the f64 pair chain evaluated on the device (`kicks_f64`).
"""

import numpy as np

from . import _abi, init
from .core import DT, ForceMode, Pair, System, Wall, box_for
from .engine import GpuEngine

NAMES = ["md_kicks_vs_cpu", "md_run_to_run", "md_reversal", "md_permutation", "md_momentum", "md_verlet_vs_cells", "md_walls_reversal",
         "md_int_golden"]

# State hash of golden_int_setup after 1000 steps with all-integer forces (checks.rs:167).
GOLDEN_INT_HASH = 0x3AAEFF680A2F0278

_M64 = (1 << 64) - 1


class SplitMix:
    """SplitMix64 (Steele, Lea and Flood, 2014), as gpu_prims::checks::SplitMix (checks.rs:14-28)."""

    def __init__(self, seed):
        self.s = seed & _M64

    def next_u64(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & _M64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def below(self, n):
        return self.next_u64() % n


def _fluid(n, pair, seed):
    """checks.rs:26-30: n particles of species 0 at density 0.6 and T 1."""
    sys_ = System(box_for(n, 0.6, 1.0), DT, pair, [1.0])
    return sys_, init.fluid(sys_, n, 1.0, seed)


def golden_setup():
    """checks.rs:33-36: 3000 WCA particles after 1000 steps."""
    sys_, s = _fluid(3000, Pair.wca(), 2026)
    return sys_, s, 1000


def golden_int_setup():
    """checks.rs:156-164: a binary LJ mixture of 3000 particles (every fourth of species 1)."""
    sys_ = System(box_for(3000, 0.6, 1.0), DT, Pair.lj(2.5), [1.0, 2.0]).with_pair(0, 1, Pair(0.7, 1.05, 2.5))
    s = init.fluid(sys_, 3000, 1.0, 2026)
    s.species[::4] = 1
    s.vel = init.maxwell(sys_, s.species, 1.0, 2026)
    return sys_, s


def kicks_vs_cpu():
    sys_, s = _fluid(3000, Pair.lj(2.5), 1)
    with GpuEngine(sys_, s) as e:
        e.step(100)
        kg, _ = e.kicks()
        k64, _ = e.kicks_f64()
    num = float(((kg.astype(np.float64) - k64) ** 2).sum())
    den = float((k64.astype(np.float64) ** 2).sum())
    rel = (num / den) ** 0.5
    if rel > 1e-5:
        return False, f"rms relative kick error vs f64 {rel:.2e}"
    return True, f"rms error of the f32 kicks vs the f64 pair chain {rel:.1e} ({len(kg)} particles)"


def run_to_run():
    sys_, s, steps = golden_setup()
    with GpuEngine(sys_, s) as a, GpuEngine(sys_, s) as b:
        a.step(steps)
        b.step(steps)
        ha, hb = a.read_state().hash(), b.read_state().hash()
    if ha != hb:
        return False, f"hashes differ: {ha:016x} vs {hb:016x}"
    return True, f"state hash after {steps} steps: {ha:016x}"


def reversal():
    sys_, s0 = _fluid(4000, Pair.wca(), 3)
    with GpuEngine(sys_, s0) as e:
        e.step(1500)
        e.reverse()
        e.step(1500)
        e.reverse()
        s = e.read_state()
    if s != s0:
        return False, "forward 1500, reverse, 1500, reverse did not restore the state"
    return True, "1500 steps forward and back restore every bit"


def permutation():
    sys_, s0 = _fluid(3000, Pair.wca(), 4)
    rng = SplitMix(4)
    perm = list(range(s0.n()))
    for i in range(len(perm) - 1, 0, -1):
        j = rng.below(i + 1)
        perm[i], perm[j] = perm[j], perm[i]
    with GpuEngine(sys_, s0) as a, GpuEngine(sys_, s0.permuted(perm)) as b:
        a.step(500)
        b.step(500)
        same = a.read_state() == b.read_state().unpermuted(perm)
    if not same:
        return False, "shuffling storage order changed the trajectory"
    return True, "shuffled storage order gives the identical trajectory"


def momentum():
    sys_, s0 = _fluid(3000, Pair.lj(2.5), 5)
    with GpuEngine(sys_, s0) as e:
        e.step(1000)
        p = e.read_state().velocity_sum()
    if p != [0, 0]:
        return False, f"integer momentum drifted to {p}"
    return True, "integer momentum exactly zero after 1000 steps"


def verlet_vs_cells():
    sys_, s0 = _fluid(5000, Pair.lj(2.5), 6)
    with GpuEngine(sys_, s0, ForceMode.cell_list()) as a, GpuEngine(sys_, s0, ForceMode.verlet_for(sys_, s0.n())) as b:
        a.step(1000)
        b.step(1000)
        rebuilds, overflow = b.read_list_stats()
        if overflow:
            return False, "neighbour list overflowed"
        if a.read_state() != b.read_state():
            return False, "Verlet-list and cell-list trajectories differ"
    return True, f"identical trajectories over 1000 steps ({rebuilds} list rebuilds, decided on the GPU)"


def walls_reversal():
    """checks.rs:132-154: hard and soft walls, gravity and a two-species pair table, reversed."""
    sys_ = (System(box_for(3000, 0.4, 1.0), DT, Pair.lj(2.5), [1.0, 3.0]).with_pair(0, 1, Pair(0.5, 1.2, 3.0))
            .with_walls(0, Wall.hard(), Wall.hard()).with_walls(1, Wall.soft(), Wall.soft()).with_gravity([0.0, -0.05]))
    s0 = init.fluid(sys_, 3000, 1.0, 7)
    s0.species[::4] = 1
    with GpuEngine(sys_, s0) as e:
        e.step(1500)
        hits = sum(e.read_ledger()[2])
        e.reverse()
        e.step(1500)
        e.reverse()
        s = e.read_state()
    if s != s0:
        return False, "walls + gravity + mixture: reversal did not restore the state"
    return True, f"exact reversal with walls ({hits} hits), gravity and a binary mixture"


def int_golden():
    sys_, s0 = golden_int_setup()
    with GpuEngine(sys_, s0, ForceMode.cell_list(), arith=_abi.ARITH_INT) as e:
        e.step(1000)
        h = e.read_state().hash()
    if h != GOLDEN_INT_HASH:
        return False, f"all-integer hash {h:016x}, golden {GOLDEN_INT_HASH:016x}"
    return True, f"all-integer forces reproduce the golden hash {h:016x}"


_CHECKS = {
    "md_kicks_vs_cpu": kicks_vs_cpu,
    "md_run_to_run": run_to_run,
    "md_reversal": reversal,
    "md_permutation": permutation,
    "md_momentum": momentum,
    "md_verlet_vs_cells": verlet_vs_cells,
    "md_walls_reversal": walls_reversal,
    "md_int_golden": int_golden,
}


def run(name):
    """checks::run (checks.rs:12-24): (True, message) or (False, message)."""
    fn = _CHECKS.get(name)
    if fn is None:
        return False, f"unknown check {name}"
    return fn()
