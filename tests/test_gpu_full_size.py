"""The engine against the oracle at the benchmark workloads' full sizes, bit for bit.

Smaller tests compare whole trajectories; here the systems are the ones the benchmark runs:
- the 3D LJ liquid, FCC N = 2^20 at rho 0.8442, T 0.72, skin 0.3: the seeded initial state,
  every particle's kick (at step 0 and step 100), the Verlet lists of a seeded sample of 10^4
  particles, a 10-step trajectory from the lattice start and one step from step 100, each against
  md-ref's IntEngine3<f32> restated (crates/md-ref/src/int_engine3.rs:48-184) and the list
  definition of crates/md/shaders/md3.wgsl:443-483;
- the 2D liquid-vapour slab, N = 2^24: the initial state, the kicks and lists of a seeded sample
  of 10^4 particles at step 0 and at step 100, and the step from 100 to 101 of that sample
  (IntEngine<f32>, crates/md-ref/src/int_engine.rs:130-344);
- the 1024 batched replicas: every replica after one 100-step graph block against IntEngine<f32>
  run on that system alone (the reference's cells-equal-Verlet invariant makes the trajectory
  independent of how the systems are stepped, crates/md/tests/gpu_engine.rs:256-273).

The oracle evaluates every kick of a million-particle system in about a second on the host's
cores; larger systems are checked on a sample."""

import concurrent.futures
import os

import numpy as np
import pytest

from micrographia_gb300 import ForceMode, GpuEngine, GpuEngine3, workloads

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
SAMPLE = 10_000


def _sample(n, seed):
    return np.sort(np.random.default_rng(seed).choice(n, min(SAMPLE, n), replace=False)).astype(np.uint32)


def _lists_match(O, g, sys_, st, skin, sample, max_total=None):
    _, offs, nbr = g.debug_list_flat(max_total)
    want = O.verlet_lists_of(sys_, st, skin, sample, THREADS)
    for q, i in enumerate(sample):
        got = np.sort(nbr[offs[i] : offs[i + 1]])
        assert np.array_equal(got, want[q]), f"particle {i}: {len(got)} listed, the oracle lists {len(want[q])}"


def test_config2_full_size_matches_the_oracle(O):
    n = 1 << 20
    sys3, spec = workloads.config2(n)
    sample = _sample(n, 2)
    with GpuEngine3(sys3, None, ForceMode.verlet_with_skin(sys3, n, 0.3), init=spec) as g:
        s0 = g.read_state()
        assert s0 == O.init(sys3, spec)
        cpu = O.IntEngine(sys3, s0, threads=THREADS)
        kg, _ = g.kicks()
        kc, _ = cpu.kicks()
        assert np.array_equal(kg, kc), f"{(kg != kc).any(axis=1).sum()} of {n} kicks differ at step 0"
        _lists_match(O, g, sys3, s0, 0.3, sample)
        g.step(10)
        cpu.step(10)
        assert g.read_state() == cpu.state
        g.step(90)
        s100 = g.read_state()
        rebuilds, overflow = g.read_list_stats()
        assert not overflow and rebuilds >= 2
        c100 = O.IntEngine(sys3, s100, threads=THREADS)
        kg, _ = g.kicks()
        kc, _ = c100.kicks()
        assert np.array_equal(kg, kc), f"{(kg != kc).any(axis=1).sum()} of {n} kicks differ at step 100"
        g.step(1)
        c100.step(1)
        assert g.read_state() == c100.state
        # lists rebuilt from the state at step 101
        g.sort_now()
        _lists_match(O, g, sys3, g.read_state(), 0.3, sample)


def test_slab_full_size_matches_the_oracle_on_a_sample(O):
    sys_, spec = workloads.config3(1 << 24)
    n = spec.n
    sample = _sample(n, 3)
    box = np.array(sys_.box_len, np.int64)
    with GpuEngine(sys_, None, ForceMode.verlet_with_skin(sys_, n, 0.3), init=spec) as g:
        s0 = g.read_state()
        assert s0 == O.init(sys_, spec)
        kg, _ = g.kicks()
        kc = O.IntEngine(sys_, s0, threads=THREADS).kicks_of(sample)
        assert np.array_equal(kg[sample], kc)
        _lists_match(O, g, sys_, s0, 0.3, sample, max_total=n * 48)
        g.step(100)
        s100 = g.read_state()
        kg, _ = g.kicks()
        kc = O.IntEngine(sys_, s100, threads=THREADS).kicks_of(sample)
        assert np.array_equal(kg[sample], kc)
        g.step(1)
        s101 = g.read_state()
        # the leapfrog of the sample (int_engine.rs:265-339, periodic, no gravity): v += kick
        # (wrapping i32), x += v, wrapped into [0, L)
        v = (s100.vel[sample].astype(np.int64) + kc).astype(np.uint32).astype(np.int32)
        x = s100.pos[sample] + v
        x = np.where(x < 0, x + box, np.where(x >= box, x - box, x))
        assert np.array_equal(s101.vel[sample], v)
        assert np.array_equal(s101.pos[sample], x)
        rebuilds, overflow = g.read_list_stats()
        assert not overflow and rebuilds >= 1


def test_config4_every_replica_matches_its_oracle_run(O):
    from micrographia_gb300 import BatchEngine

    cfg = workloads.config4()
    systems = [s for s, _ in cfg]
    states = [O.init(s, spec) for s, spec in cfg]
    with BatchEngine(systems, states, ForceMode.verlet_with_skin(None, 0, 0.3), block_steps=100) as b:
        b.step(100)
        launches, rebuilds = b.stats()
        assert rebuilds >= 2
        got = [b.read_system(k) for k in range(len(systems))]

    def same(k):
        c = O.IntEngine(systems[k], states[k])
        c.step(100)
        return c.state == got[k]

    # largest systems first; the oracle's calls release the interpreter lock
    order = sorted(range(len(systems)), key=lambda k: -states[k].n())
    with concurrent.futures.ThreadPoolExecutor(THREADS) as ex:
        ok = dict(zip(order, ex.map(same, order)))
    bad = [k for k in range(len(systems)) if not ok[k]]
    assert not bad, f"{len(bad)} of {len(systems)} replicas differ from their oracle runs, first {bad[:8]}"


def test_config2_energy_is_conserved_at_full_size():
    """The 3D LJ liquid of configs[1] at full size (N = 2^20, rho 0.8442, T 0.72, skin 0.3):
    after 1000 steps of equilibration from the lattice, the total energy per atom (on-step
    kinetic + pair potential, FP64 sums) stays within the reference's bar of 2e-3 over 5000
    steps (md/tests/three.rs:95-111), and its least-squares slope is below 1e-8 per atom per step:
    the integer leapfrog is exactly time-reversible, so what remains is the f32 force error."""
    n = 1 << 20
    sys3, spec = workloads.config2(n)
    with GpuEngine3(sys3, None, ForceMode.verlet_with_skin(sys3, n, 0.3), init=spec) as g:
        g.step(1000)
        e = []
        for _ in range(26):
            ke, pe = g.energy()
            e.append((ke + pe) / n)
            g.step(200)
    e = np.array(e)
    slope = np.polyfit(np.arange(e.size) * 200.0, e, 1)[0]
    assert e.max() - e.min() < 2e-3, (e.max() - e.min())
    assert abs(slope) < 1e-8, slope
