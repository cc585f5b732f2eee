"""Half-shell lists (3D, one species): each pair listed and evaluated once, its kick mirrored onto
the other particle (crates/md-ref/src/fast.rs:240-246 rounds the two ends the same way).

Bit-exact bars against the oracle (md-ref's IntEngine3<f32> restated): the lists, read back as both
ends' neighbour sets, equal the list definition of crates/md/shaders/md3.wgsl:443-483; kicks and
trajectories equal IntEngine3<f32>'s (int_engine3.rs:48-184), including overlapping pairs whose
kicks saturate the i32 conversion; and the engine with half lists equals the same engine with full
lists."""

import numpy as np
import pytest

from micrographia_gb300 import ForceMode, GpuEngine3, Pair, State3, System3, _abi, cube_for

pytestmark = pytest.mark.gpu

HALF = _abi.FLAG_HALF_LISTS
FULL = 0  # full lists: the default


def liquid3(O, n, density, t, seed=3):
    sys3 = System3(cube_for(n, density), 0.005, Pair.lj(2.5), [1.0])
    return sys3, O.fcc_maxwell(sys3, n, t, seed, jitter=0.05)


@pytest.mark.parametrize("n,density", [(4000, 0.8442), (50_000, 0.8442), (20_000, 0.3)])
def test_half_lists_give_the_oracle_neighbour_sets(O, n, density):
    sys3, st = liquid3(O, n, density, 1.0, seed=n)
    cpu = O.IntEngine(sys3, st)
    cpu.step(30)
    st = cpu.state
    with GpuEngine3(sys3, st, ForceMode.verlet_with_skin(sys3, n, 0.3), flags=HALF) as g:
        got = g.debug_list()
    want = O.verlet_lists(sys3, st, 0.3)
    assert [len(x) for x in got] == [len(x) for x in want]
    assert np.array_equal(np.concatenate(got), np.concatenate(want))


@pytest.mark.parametrize("n,t,steps", [(4000, 1.0, 300), (6000, 6.0, 200), (60_000, 0.72, 120)])
def test_half_lists_follow_the_oracle(O, n, t, steps):
    sys3, st = liquid3(O, n, 0.8442, t)
    with GpuEngine3(sys3, st, ForceMode.verlet_with_skin(sys3, n, 0.3), flags=HALF) as g:
        g.step(steps)
        got = g.read_state()
        rebuilds, overflow = g.read_list_stats()
        kg, _ = g.kicks()
    assert not overflow and rebuilds >= 2
    cpu = O.IntEngine(sys3, st, threads=8)
    cpu.step(steps)
    assert got == cpu.state
    kc, _ = cpu.kicks()
    assert np.array_equal(kg, kc)


def test_half_and_full_lists_give_the_same_trajectory(O):
    n = 300_000
    sys3, st = liquid3(O, n, 0.8442, 0.72)
    out = {}
    for name, flags in [("half", HALF), ("full", FULL)]:
        with GpuEngine3(sys3, st, ForceMode.verlet_with_skin(sys3, n, 0.3), flags=flags) as g:
            g.step(150)
            out[name] = g.read_state()
    assert out["half"] == out["full"]


@pytest.mark.parametrize("sep", [0.05, 0.3])
def test_half_lists_with_saturated_kicks(O, sep):
    """Two particles `sep` sigma apart (0.05: the chain with the library's division, below
    sigma / 8; 0.3: the packed chain): a * f overflows the i32 conversion, which saturates (Rust's
    `as`); the mirrored kick must saturate the other way, not wrap."""
    n = 4000
    sys3, st = liquid3(O, n, 0.8442, 1.0)
    pos = st.pos.copy()
    pos[1] = pos[0] + np.array([int(0.8 * sep * 2**32), int(0.6 * sep * 2**32), 0], np.int64)
    pos[1] %= np.array(sys3.box_len, np.int64)
    st = State3(pos, st.vel.copy(), st.species.copy())
    cpu = O.IntEngine(sys3, st)
    kc, _ = cpu.kicks()
    # the case this test is for: the pair's kicks saturate (the particles' other kicks are small)
    assert (np.abs(kc[:2, :2].astype(np.int64)) > 2**31 - 2**21).all()
    with GpuEngine3(sys3, st, ForceMode.verlet_with_skin(sys3, n, 0.3), flags=HALF) as g:
        g.step(1)
        got = g.read_state()
    cpu.step(1)
    assert got == cpu.state


def test_half_lists_reverse_exactly(O):
    n = 8000
    sys3, st = liquid3(O, n, 0.8442, 1.0)
    with GpuEngine3(sys3, st, ForceMode.verlet_with_skin(sys3, n, 0.3), flags=HALF) as g:
        h0 = g.state_hash()
        g.step(150)
        g.reverse()
        g.step(150)
        g.reverse()
        assert g.state_hash() == h0
