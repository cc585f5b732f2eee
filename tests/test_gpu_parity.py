"""The CUDA engine against the oracle (md-ref's CPU engine restated), through the C ABI.

Bit-exact bars: initial conditions, cell keys / starts / the stable sort permutation, Verlet lists
(as neighbour sets), per-particle kicks and integer trajectories against IntEngine<f32> /
IntEngine3<f32>. Tolerance bars (written at each assert): energies against the f64 engine.
Reference tests mirrored: crates/md/tests/gpu_engine.rs, three.rs, crates/md/src/checks.rs,
crates/gpu-prims/src/checks.rs."""

import math
import os

import numpy as np
import pytest

from micrographia_gb300 import ONE, ForceMode, GpuEngine, GpuEngine3, Pair, State, State3, System, System3, box_for, cube_for
from micrographia_gb300 import _abi
from micrographia_gb300.engine import init_state, make_init

pytestmark = pytest.mark.gpu


def fluid(O, n, density, pair, seed, t=1.0):
    sys_ = System(box_for(n, density, 1.0), 0.005, pair, [1.0])
    return sys_, O.fluid(sys_, n, t, seed)


def equilibrated(O, n, density, pair, seed, steps=200):
    sys_, s = fluid(O, n, density, pair, seed)
    e = O.IntEngine(sys_, s)
    e.step(steps)
    return sys_, e.state


def liquid3(O, n, density, t, seed=3):
    sys3 = System3(cube_for(n, density), 0.005, Pair.lj(2.5), [1.0])
    return sys3, O.fcc_maxwell(sys3, n, t, seed, jitter=0.05)


# ---------------------------------------------------------------- initial conditions
@pytest.mark.parametrize(
    "recipe,dim,n,args",
    [
        (_abi.INIT_FLUID, 2, 3000, dict(t=1.0, seed=2026, jitter=0.1)),
        (_abi.INIT_FLUID, 2, 1, dict(t=1.0, seed=5, jitter=0.1)),
        (_abi.INIT_TRIANGULAR, 2, 4096, dict(t=0.8, seed=1, jitter=0.1)),
        (_abi.INIT_FCC, 3, 4000, dict(t=1.0, seed=3, jitter=0.05)),
        (_abi.INIT_FCC, 3, 4 * 8**3, dict(t=0.72, seed=1, jitter=0.05)),
        (_abi.INIT_SLAB, 2, 20000, dict(t=0.45, seed=7, jitter=0.1)),
    ],
)
def test_seeded_init_is_bit_identical(O, recipe, dim, n, args):
    if dim == 2:
        rho = 0.2125 if recipe == _abi.INIT_SLAB else 0.7
        sys_ = System(box_for(n, rho, 4.0 if recipe == _abi.INIT_SLAB else 1.0), 0.005, Pair.lj(2.5), [1.0])
    else:
        sys_ = System3(cube_for(n, 0.8442), 0.005, Pair.lj(2.5), [1.0])
    spec = make_init(recipe, n, args["t"], args["seed"], args["jitter"], 0.7, 0.05, 0.25)
    want = O.init(sys_, spec)
    got = init_state(sys_, recipe, n, args["t"], args["seed"], args["jitter"], 0.7, 0.05, 0.25)
    assert np.array_equal(got.pos, want.pos)
    assert np.array_equal(got.vel, want.vel)
    assert np.array_equal(got.species, want.species)
    assert got.velocity_sum() == [0] * dim


@pytest.mark.parametrize("walls", [(0,), (1,), (0, 1)])
def test_seeded_fluid_with_walls_is_bit_identical(O, walls):
    """init::fluid (init.rs:105-121) in a box with walls: on each walled axis the lattice fills
    the box less 2 sigma and sits 1 sigma clear of the walls; the triangular and slab recipes
    refuse walled boxes."""
    from micrographia_gb300 import Wall

    n = 2500
    sys_ = System(box_for(n, 0.5, 1.3), 0.005, Pair.lj(2.5), [1.0])
    for a in walls:
        sys_.with_walls(a, Wall.soft(), Wall.hard())
    spec = make_init(_abi.INIT_FLUID, n, 1.0, 11, 0.1, 0.7, 0.05, 0.25)
    want = O.init(sys_, spec)
    got = init_state(sys_, _abi.INIT_FLUID, n, 1.0, 11, 0.1)
    assert np.array_equal(got.pos, want.pos)
    assert np.array_equal(got.vel, want.vel)
    for a in walls:
        assert got.pos[:, a].min() >= ONE and got.pos[:, a].max() < sys_.box_len[a] - ONE
    for recipe in (_abi.INIT_TRIANGULAR, _abi.INIT_SLAB):
        with pytest.raises(RuntimeError):
            init_state(sys_, recipe, n, 1.0, 11)


@pytest.mark.parametrize("dim", [2, 3])
def test_maxwell_for_given_species_is_bit_identical(O, dim):
    """init::maxwell (init.rs:42-57) / three::maxwell for a species pattern with three masses and
    (3D) a pinned species: equal to the oracle's draw, velocity sums exactly zero."""
    from micrographia_gb300 import init

    n = 3001
    if dim == 2:
        sys_ = System(box_for(n, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0, 2.0, 0.5])
    else:
        sys_ = System3(cube_for(n, 0.8), 0.005, Pair.lj(2.5), [1.0, 2.0, 0.5])
        sys_.with_pinned(2)
    sp = (np.arange(n) % 3).astype(np.uint32)
    got = init.maxwell(sys_, sp, 0.9, 2026)
    assert np.array_equal(got, O.maxwell(sys_, sp, 0.9, 2026))
    moving = ~((sys_.pinned >> sp) & 1).astype(bool) if dim == 3 else np.ones(n, bool)
    assert (got[moving].astype(np.int64).sum(axis=0) == 0).all()


def test_libm_restatement_on_device_matches_over_many_draws(O):
    """Millions of Box–Muller draws (log, cos): the device velocities equal the oracle's."""
    n = 1 << 20
    sys3 = System3(cube_for(n, 0.8442), 0.005, Pair.lj(2.5), [1.0])
    got = init_state(sys3, _abi.INIT_FCC, n, 0.72, 12345, 0.05)
    want = O.init(sys3, make_init(_abi.INIT_FCC, n, 0.72, 12345, 0.05))
    assert np.array_equal(got.vel, want.vel)
    assert np.array_equal(got.pos, want.pos)


def test_velocity_rescale_integer_arithmetic():
    """The thermostat's v <- round(v f) as i32 in integers (the exact product rounded as the f64
    multiply rounds it, then half away from zero) equals the f64 product and rounding on 2^26
    seeded random cases: extreme and tiny velocities, factors near 1, wide exponents, ties."""
    import ctypes as C

    checked, bad = C.c_uint64(), C.c_uint64()
    _abi.check(_abi.lib().gbmd_check_rescale(1 << 26, 0, C.byref(checked), C.byref(bad)))
    assert checked.value == 1 << 26
    assert bad.value == 0, bad.value


def test_device_libm_equals_the_oracle_fdlibm(O):
    """The device's ln, cos and sin (the initial velocities', heat bath's and thermal walls' draws)
    equal the oracle's fdlibm restatement bit for bit on 4 x 10^6 arguments: the bath's own
    ranges (1 - U in (0, 1], 2 pi U), and wider ones (cos and sin up to 10^6, where the argument
    reduction takes more terms; ln from 1e-304 to 1e304, and negative arguments)."""
    import ctypes as C

    rng = np.random.default_rng(77)
    parts = [
        1.0 - rng.random(1_000_000),
        6.283185307179586 * rng.random(1_000_000),
        rng.uniform(-1e6, 1e6, 1_000_000),
        np.exp(rng.uniform(-700, 700, 1_000_000)) * rng.choice([-1.0, 1.0], 1_000_000),
    ]
    x = np.ascontiguousarray(np.concatenate(parts))
    got = np.empty((x.size, 3), np.float64)
    _abi.check(_abi.lib().gbmd_debug_libm(x.ctypes.data_as(C.POINTER(C.c_double)), x.size, got.ctypes.data_as(C.POINTER(C.c_double))))
    want = O.fdlibm_many(x)
    same = (got.view(np.uint64) == want.view(np.uint64)) | (np.isnan(got) & np.isnan(want))
    same[np.abs(x) >= 1e6, 1:] = True  # (cos and sin: the restatement reduces |x| < 2^20 pi/2 only)
    assert same.all(), (x[~same.all(1)][:5], got[~same.all(1)][:5], want[~same.all(1)][:5])


# ---------------------------------------------------------------- binning (gpu-prims checks.rs:30-149)
SIZES = [1, 2, 255, 256, 257, 1023, 1024, 1025, 4097, 65537, (1 << 20) + 3]


@pytest.mark.parametrize("n", SIZES)
def test_binning_matches_cell_list(O, n):
    rng = np.random.default_rng(n)
    sys_ = System(box_for(max(n, 200), 0.7, 1.0), 0.005, Pair.lj(2.5), [1.0])
    pos = np.stack([rng.integers(0, sys_.box_len[a], n) for a in range(2)], 1).astype(np.int64)
    st = State(pos, np.zeros((n, 2), np.int32), np.zeros(n, np.uint32))
    dims = sys_.cells_for(2.5)
    with GpuEngine(sys_, st, ForceMode.cell_list()) as e:
        keys, start, items, order = e.debug_bin(dims)
    assert np.array_equal(order, np.arange(n))
    wk, ws, wi = O.cell_list(sys_, st, dims)
    assert np.array_equal(keys, wk)
    assert np.array_equal(start, ws)
    assert np.array_equal(items, wi)


def test_binning_all_one_key(O):
    n = 300_001
    sys_ = System(box_for(n, 0.7, 1.0), 0.005, Pair.lj(2.5), [1.0])
    pos = np.full((n, 2), ONE // 3, np.int64)
    pos[:, 0] += np.arange(n) % 1000
    st = State(pos, np.zeros((n, 2), np.int32), np.zeros(n, np.uint32))
    dims = sys_.cells_for(2.5)
    with GpuEngine(sys_, st, ForceMode.cell_list()) as e:
        keys, start, items, _ = e.debug_bin(dims)
    wk, ws, wi = O.cell_list(sys_, st, dims)
    assert np.array_equal(keys, wk) and np.array_equal(start, ws) and np.array_equal(items, wi)


def test_binning_3d(O):
    sys3, st = liquid3(O, 32000, 0.8442, 0.72)
    dims = sys3.cells_for(2.8)
    with GpuEngine3(sys3, st) as e:
        keys, start, items, _ = e.debug_bin(dims)
    wk, ws, wi = O.cell_list(sys3, st, dims)
    assert np.array_equal(keys, wk) and np.array_equal(start, ws) and np.array_equal(items, wi)


# ---------------------------------------------------------------- Verlet lists
def test_verlet_lists_match_2d(O):
    sys_, st = equilibrated(O, 3000, 0.7, Pair.lj(2.5), 1, steps=50)
    with GpuEngine(sys_, st, ForceMode.verlet_with_skin(sys_, 3000, 0.3)) as e:
        got = e.debug_list()
    want = O.verlet_lists(sys_, st, 0.3)
    for i in range(st.n()):
        assert np.array_equal(got[i], want[i]), i


def test_verlet_lists_match_3d(O):
    sys3, st = liquid3(O, 4000, 0.8442, 0.72)
    with GpuEngine3(sys3, st, ForceMode.verlet_with_skin(sys3, 4000, 0.3)) as e:
        got = e.debug_list()
    want = O.verlet_lists(sys3, st, 0.3)
    for i in range(st.n()):
        assert np.array_equal(got[i], want[i]), i


@pytest.mark.parametrize(
    "dim,n,flags",
    [
        (3, 4000, 0),
        (3, 4000, _abi.FLAG_WHOLE_CELLS),
        (3, 50000, _abi.build_lanes_flag(1)),
        (3, 50000, _abi.build_lanes_flag(4)),
        (3, 50000, _abi.build_lanes_flag(8) | _abi.FLAG_WHOLE_CELLS),
        (3, 250000, 0),
        (2, 20000, _abi.build_lanes_flag(8)),
        (2, 120000, 0),
    ],
)
def test_verlet_lists_across_build_variants(O, dim, n, flags):
    """Every list build (cells stored by slabs of the last axis or whole; 1, 2, 4 or 8 lanes per
    particle) gives the oracle's neighbour sets."""
    if dim == 3:
        sys_, st = liquid3(O, n, 0.8442, 1.0, seed=n)
        eng = GpuEngine3
    else:
        sys_, st = fluid(O, n, 0.7, Pair.lj(2.5), n % 997)
        eng = GpuEngine
    with eng(sys_, st, ForceMode.verlet_with_skin(sys_, n, 0.3), flags=flags) as e:
        got = e.debug_list()
    want = O.verlet_lists(sys_, st, 0.3)
    assert [len(g) for g in got] == [len(w) for w in want]
    assert np.array_equal(np.concatenate(got), np.concatenate(want))


# ---------------------------------------------------------------- kicks (gpu_engine.rs:27-60; three.rs:33-64)
@pytest.mark.parametrize("pair", [Pair.wca(), Pair.lj(2.5)])
@pytest.mark.parametrize("mode", ["cells", "verlet"])
def test_kicks_are_bit_identical_2d(O, pair, mode):
    sys_, s = equilibrated(O, 3000, 0.7, pair, 1)
    m = ForceMode.cell_list() if mode == "cells" else ForceMode.verlet_for(sys_, 3000)
    with GpuEngine(sys_, s, m) as g:
        kg, peg = g.kicks()
    k32, pe32 = O.IntEngine(sys_, s).kicks()
    k64, _ = O.IntEngine(sys_, s, f64=True).kicks()
    assert np.array_equal(kg, k32), f"{(kg != k32).any(axis=1).sum()} kicks differ"
    rel64 = math.sqrt(((kg.astype(np.float64) - k64) ** 2).sum() / (k64.astype(np.float64) ** 2).sum())
    assert rel64 < 1e-5  # md-ref physics.rs:144
    assert abs((peg - pe32) / pe32) < 1e-5  # f64 sum of the same f32 pair energies, other order


def test_kicks_are_bit_identical_3d(O):
    sys3, s = liquid3(O, 4000, 0.8, 1.0)
    cpu = O.IntEngine(sys3, s)
    cpu.step(100)
    st = cpu.state
    with GpuEngine3(sys3, st) as g:
        kg, peg = g.kicks()
    kc, pec = cpu.kicks()
    k64, _ = O.IntEngine(sys3, st, f64=True).kicks()
    assert np.array_equal(kg, kc)
    rel64 = math.sqrt(((kg.astype(np.float64) - k64) ** 2).sum() / (k64.astype(np.float64) ** 2).sum())
    assert rel64 < 1e-5
    assert abs((peg - pec) / pec) < 1e-5


def test_kicks_binary_mixture(O):
    sys_ = System(box_for(3000, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0, 3.0]).with_pair(0, 1, Pair(0.6, 1.1, 2.5))
    s = O.fluid(sys_, 3000, 1.0, 1)
    s.species[::3] = 1
    s.vel = O.maxwell(sys_, s.species, 1.0, 1)
    cpu = O.IntEngine(sys_, s)
    cpu.step(100)
    st = cpu.state
    for mode in (ForceMode.cell_list(), ForceMode.verlet_for(sys_, 3000)):
        with GpuEngine(sys_, st, mode) as g:
            kg, _ = g.kicks()
        assert np.array_equal(kg, cpu.kicks()[0])


# ---------------------------------------------------------------- trajectories
def test_trajectory_is_bit_identical_2d_cells(O):
    sys_, s0 = fluid(O, 2000, 0.6, Pair.wca(), 7)
    with GpuEngine(sys_, s0, ForceMode.cell_list()) as g:
        c = O.IntEngine(sys_, s0)
        for _ in range(4):
            g.step(50)
            c.step(50)
            assert g.read_state() == c.state


def test_trajectory_is_bit_identical_2d_verlet(O):
    sys_, s0 = fluid(O, 4096, 0.7, Pair.lj(2.5), 11, t=0.8)
    with GpuEngine(sys_, s0, ForceMode.verlet_with_skin(sys_, 4096, 0.3)) as g:
        c = O.IntEngine(sys_, s0)
        g.step(333)
        c.step(333)
        assert g.read_state() == c.state
        rebuilds, overflow = g.read_list_stats()
        assert not overflow and rebuilds > 1


def test_trajectory_is_bit_identical_3d_verlet(O):
    sys3, s0 = liquid3(O, 4000, 0.8442, 0.72)
    with GpuEngine3(sys3, s0, ForceMode.verlet_with_skin(sys3, 4000, 0.3)) as g:
        c = O.IntEngine(sys3, s0)
        g.step(120)
        c.step(120)
        assert g.read_state() == c.state


@pytest.mark.parametrize(
    "dim,n,lanes",
    [(3, 65536, 2), (3, 200_000, 2), (3, 262144, 1), (2, 300_000, 1), (2, 65535, 4)],
)
def test_trajectory_across_lane_splits(O, dim, n, lanes):
    """The force kernel gives each particle 4, 2 or 1 lanes by system size (below 65536, 262144,
    else); every variant, through list rebuilds, follows IntEngine's trajectory bit for bit."""
    if dim == 3:
        sys_, s0 = liquid3(O, n, 0.8442, 1.2, seed=n)
    else:
        sys_, s0 = fluid(O, n, 0.7, Pair.lj(2.5), n % 1000, t=1.2)
    eng = GpuEngine3 if dim == 3 else GpuEngine
    with eng(sys_, s0, ForceMode.verlet_with_skin(sys_, n, 0.3)) as g:
        c = O.IntEngine(sys_, s0, threads=min(16, os.cpu_count() or 1))
        g.step(40)
        c.step(40)
        assert g.read_state() == c.state
        rebuilds, overflow = g.read_list_stats()
        assert not overflow and rebuilds > 1


@pytest.mark.parametrize(
    "dim,n,lanes", [(3, 4000, 0), (3, 4000, 16), (2, 20000, 0), (2, 9000, 16), (3, 60_000, 0), (3, 90_000, 1)]
)
def test_step_loop_follows_the_oracle(O, dim, n, lanes):
    """Small systems step in a persistent loop (a cooperative launch per run of steps between
    list rebuilds), with 1 to 16 lanes per particle: 200 steps (three 64-step blocks and single
    steps) equal IntEngine's."""
    if dim == 3:
        sys_, s0 = liquid3(O, n, 0.8442, 1.2, seed=n + 1)
        eng = GpuEngine3
    else:
        sys_, s0 = fluid(O, n, 0.7, Pair.lj(2.5), 5, t=1.2)
        eng = GpuEngine
    with eng(sys_, s0, ForceMode.verlet_with_skin(sys_, n, 0.3), flags=_abi.force_lanes_flag(lanes)) as g:
        c = O.IntEngine(sys_, s0, threads=min(16, os.cpu_count() or 1))
        g.step(200)
        c.step(200)
        assert g.read_state() == c.state
        rebuilds, overflow = g.read_list_stats()
        assert not overflow and rebuilds > 3


@pytest.mark.parametrize("dim,n,t", [(3, 8000, 1.0), (2, 30000, 1.0), (3, 6000, 6.0)])
def test_step_loop_equals_per_step_graphs(O, dim, n, t):
    """The loop and the per-step graph nodes give the same state and the same rebuilds over 1000
    steps, also when a hot fluid rebuilds every few steps; two engines alive at once both step
    through per-step graphs."""
    if dim == 3:
        sys_, s0 = liquid3(O, n, 0.8442, t, seed=7)
        eng = GpuEngine3
    else:
        sys_, s0 = fluid(O, n, 0.7, Pair.lj(2.5), 9, t=t)
        eng = GpuEngine
    mode = ForceMode.verlet_with_skin(sys_, n, 0.3)
    runs = []
    for flags in (0, _abi.FLAG_NO_STEP_LOOP):  # one engine at a time: the loop runs for a lone engine
        with eng(sys_, s0, mode, flags=flags) as g:
            g.step(1000)
            runs.append((g.read_state().hash(), g.read_list_stats(), g.launch_count()))
    (ha, ra, la), (hb, rb, lb) = runs
    assert ha == hb
    assert ra == rb and ra[0] > 10
    assert la < lb
    with eng(sys_, s0, mode) as a, eng(sys_, s0, mode) as b:
        a.step(1000)
        b.step(1000)
        assert a.read_state().hash() == ha and a.launch_count() == lb


def test_config1_triangular_4096_1000_steps(O):
    """2D LJ N=4096, rho 0.70, triangular start, T=0.8, seed 1, cell list, 1000 steps: the GPU
    state equals md-ref's IntEngine<f32> bit for bit."""
    sys_ = System(box_for(4096, 0.7, 1.0), 0.005, Pair.lj(2.5), [1.0])
    s0 = O.init(sys_, make_init(_abi.INIT_TRIANGULAR, 4096, 0.8, 1, 0.1))
    with GpuEngine(sys_, s0, ForceMode.cell_list()) as g:
        c = O.IntEngine(sys_, s0)
        g.step(1000)
        c.step(1000)
        assert g.read_state().hash() == c.hash()


# ---------------------------------------------------------------- exactness properties (gpu_engine.rs:62-132, 256-273)
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("n", [1, 2, 5])
def test_a_few_particles_follow_the_oracle(O, dim, n):
    """The smallest systems (one particle, one pair, five) in a 12-sigma box, cell lists and
    Verlet lists: 400 steps equal the oracle's bit for bit, kicks too, and reverse exactly."""
    rng = np.random.default_rng(n)
    L = int(12 * ONE)
    if dim == 2:
        sys_ = System([L, L], 0.005, Pair.lj(2.5), [1.0])
        eng, S = GpuEngine, State
    else:
        sys_ = System3([L, L, L], 0.005, Pair.lj(2.5), [1.0])
        eng, S = GpuEngine3, State3
    pos = np.zeros((n, dim), np.int64)
    for k in range(n):
        pos[k] = (np.array([1.5 + 1.15 * k, 6.0, 6.0][:dim]) * ONE).astype(np.int64)
    vel = rng.integers(-(2**22), 2**22, (n, dim)).astype(np.int32)
    vel -= (vel.sum(axis=0) // n).astype(np.int32)
    s0 = S(pos, vel, np.zeros(n, np.uint32))
    for m in (ForceMode.cell_list(), ForceMode.verlet_with_skin(sys_, n, 0.3)):
        c = O.IntEngine(sys_, s0)
        with eng(sys_, s0, m) as g:
            g.step(400)
            c.step(400)
            assert g.read_state() == c.state
            assert np.array_equal(g.kicks()[0], c.kicks()[0])
            g.reverse()
            g.step(400)
            g.reverse()
            assert g.read_state() == s0


@pytest.mark.parametrize("loop", [False, True])
def test_path_bound_fires_the_trigger_at_the_same_steps(O, loop):
    """2D Verlet lists with the path bound (the displacement test skipped while a particle's path
    since the list build cannot reach half the skin) against the same engine testing every
    particle every step: the same rebuild count after every chunk of steps and the same states,
    through a kick to a region, a flipped bit and a reversal. `loop`: the persistent step loop,
    else per-step graph nodes."""
    n = 20000
    sys_ = System(box_for(n, 0.7, 1.0), 0.005, Pair.lj(2.5), [1.0])
    s0 = O.fluid(sys_, n, 1.0, 12)
    m = ForceMode.verlet_with_skin(sys_, n, 0.3)
    L = sys_.box_f64()
    f = 0 if loop else _abi.FLAG_NO_STEP_LOOP
    with GpuEngine(sys_, s0, m, flags=f) as a, GpuEngine(sys_, s0, m, flags=f | _abi.FLAG_NO_PATH_BOUND) as b:
        for k in range(60):
            a.step(7)
            b.step(7)
            assert a.read_list_stats() == b.read_list_stats(), k
            if k == 20:
                for e in (a, b):
                    e.kick_region([0.0, 0.0], [0.3 * L[0], L[1]], 0.0, [2.0, 0.0])
            if k == 35:
                for e in (a, b):
                    e.flip_bit(5, 0, 30)
            if k == 45:
                for e in (a, b):
                    e.reverse()
        assert a.read_state() == b.read_state()
        assert a.read_list_stats()[0] > 20


def test_run_to_run_identical(O):
    sys_, s = fluid(O, 5000, 0.6, Pair.wca(), 2)
    hs = []
    for _ in range(2):
        with GpuEngine(sys_, s, ForceMode.verlet_for(sys_, 5000)) as g:
            g.step(500)
            hs.append(g.read_state().hash())
    assert hs[0] == hs[1] and hs[0] != s.hash()


@pytest.mark.parametrize("mode", ["cells", "verlet"])
def test_reversal_is_exact(O, mode):
    sys_, s0 = fluid(O, 5000, 0.6, Pair.wca(), 3)
    m = ForceMode.cell_list() if mode == "cells" else ForceMode.verlet_for(sys_, 5000)
    with GpuEngine(sys_, s0, m) as g:
        g.step(800)
        g.reverse()
        g.step(800)
        g.reverse()
        assert g.read_state().hash() == s0.hash()
        assert g.steps == 0


def test_one_bit_flip_breaks_reversal(O):
    sys_, s0 = fluid(O, 5000, 0.6, Pair.wca(), 4)
    with GpuEngine(sys_, s0, ForceMode.verlet_for(sys_, 5000)) as g:
        g.step(2000)
        g.flip_bit(17, 0, 0)
        g.reverse()
        g.step(2000)
        g.reverse()
        differ, _ = g.read_state().position_difference(s0, sys_)
    assert differ > 4000


def test_storage_order_does_not_matter(O):
    sys_, s0 = fluid(O, 4000, 0.6, Pair.wca(), 5)
    perm = np.random.default_rng(5).permutation(4000)
    with GpuEngine(sys_, s0, ForceMode.verlet_for(sys_, 4000)) as a, GpuEngine(sys_, s0.permuted(perm), ForceMode.verlet_for(sys_, 4000)) as b:
        a.step(500)
        b.step(500)
        assert a.read_state().hash() == b.read_state().unpermuted(perm).hash()


def test_momentum_is_exactly_conserved(O):
    sys_, s0 = fluid(O, 4000, 0.6, Pair.lj(2.5), 6)
    with GpuEngine(sys_, s0, ForceMode.verlet_for(sys_, 4000)) as g:
        g.step(1000)
        assert g.read_state().velocity_sum() == [0, 0]


@pytest.mark.parametrize("pair,density", [(Pair.wca(), 0.6), (Pair.lj(2.5), 0.7)])
def test_cell_list_and_verlet_lists_give_identical_trajectories(O, pair, density):
    sys_, s0 = fluid(O, 6000, density, pair, 10)
    with GpuEngine(sys_, s0, ForceMode.cell_list()) as a, GpuEngine(sys_, s0, ForceMode.verlet_for(sys_, 6000)) as b:
        a.step(1500)
        b.step(1500)
        rebuilds, overflow = b.read_list_stats()
        assert not overflow and 1 < rebuilds < 1500
        assert a.read_state().hash() == b.read_state().hash()


def test_3d_cells_equal_verlet(O):
    sys3, s0 = liquid3(O, 6000, 0.8, 1.0)
    with GpuEngine3(sys3, s0, ForceMode.cell_list()) as a, GpuEngine3(sys3, s0) as b:
        a.step(1000)
        b.step(1000)
        assert a.read_state().hash() == b.read_state().hash()
        assert b.read_list_stats()[0] > 10


def test_upload_and_counters(O):
    sys_, s0 = fluid(O, 3000, 0.6, Pair.lj(2.5), 8)
    with GpuEngine(sys_, s0, ForceMode.verlet_for(sys_, 3000)) as g:
        g.step(100)
        mid = g.read_state()
        g.step(7)
        g.upload(mid)
        g.step(7)
        c = O.IntEngine(sys_, mid)
        c.step(7)
        assert g.read_state() == c.state
        assert g.steps == 114


# ---------------------------------------------------------------- energies and instruments
def test_energy_is_conserved_wca(O):
    """gpu_engine.rs:166-183: drift < 2e-3 per particle (against the f64 CPU energy)."""
    sys_, s0 = fluid(O, 4000, 0.6, Pair.wca(), 8)
    with GpuEngine(sys_, s0, ForceMode.verlet_for(sys_, 4000)) as g:
        g.step(500)
        energy = lambda s: sum(O.IntEngine(sys_, s, f64=True).energy()) / s.n()
        e0 = energy(g.read_state())
        worst = 0.0
        for _ in range(5):
            g.step(1000)
            worst = max(worst, abs(energy(g.read_state()) - e0))
    assert worst < 2e-3


def test_frame_matches_oracle(O):
    sys_, s = equilibrated(O, 3000, 0.7, Pair.lj(2.5), 4)
    ke64, pe64 = O.IntEngine(sys_, s, f64=True).energy()
    pe32, w32 = O.pair_sums(sys_, s)
    with GpuEngine(sys_, s, ForceMode.verlet_for(sys_, 3000)) as g:
        f, rdf, prof = g.observe(rdf_bins=200, rdf_rmax=5.0, profile_bins=80, profile_axis=0)
        ke, pe = g.energy()
    assert abs(f.potential - pe32) < 1e-9 * abs(pe32)  # same f32 terms, f64 sums in another order
    assert abs(f.virial - w32) < 1e-9 * abs(w32)
    assert abs(f.kinetic - ke64) < 1e-9 * ke64  # on-step KE from the same integer velocities
    assert abs(f.potential - pe64) < 1e-5 * abs(pe64)  # f32 pair terms against the f64 engine
    n, vol = 3000, sys_.volume()
    assert abs(f.temperature - f.kinetic / (n - 1)) < 1e-12
    assert abs(f.pressure - (n / vol * f.temperature + f.virial / (2 * vol))) < 1e-9
    assert np.array_equal(rdf, O.rdf(sys_, s, 200, 5.0))
    assert np.array_equal(prof, O.profile(sys_, s, 80, 0))
    assert (ke, pe) == (f.kinetic, f.potential)


def test_frame_3d(O):
    sys3, s = liquid3(O, 4000, 0.8442, 0.72)
    pe32, w32 = O.pair_sums(sys3, s)
    with GpuEngine3(sys3, s) as g:
        f, rdf, _ = g.observe(rdf_bins=200, rdf_rmax=5.0)
    assert abs(f.potential - pe32) < 1e-9 * abs(pe32)
    assert abs(f.virial - w32) < 1e-9 * abs(w32)
    assert np.array_equal(rdf, O.rdf(sys3, s, 200, 5.0))


@pytest.mark.parametrize("dim", [2, 3])
def test_read_kinetic_in_id_order(O, dim):
    """GpuEngine3::read_kinetic / read_kinetic_total (engine3.rs:626-637): per-particle kinetic
    energies from the half-step velocities, with their species, in id order, after the storage
    order has been shuffled by list builds; a two-species mixture (masses 1 and 2.5)."""
    if dim == 2:
        sys_ = System(box_for(2000, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0, 2.5])
        s0 = O.fluid(sys_, 2000, 1.0, 5)
        eng, mode = GpuEngine, ForceMode.verlet_with_skin(sys_, 2000, 0.3)
    else:
        sys_ = System3(cube_for(2048, 0.8442), 0.005, Pair.lj(2.5), [1.0, 2.5])
        s0 = O.fcc_maxwell(sys_, 2048, 0.72, 3, jitter=0.05)
        eng, mode = GpuEngine3, ForceMode.verlet_with_skin(sys_, 2048, 0.3)
    sp = (np.arange(s0.n()) % 3 == 0).astype(np.uint32)
    s0 = type(s0)(s0.pos, s0.vel, sp)
    c = O.IntEngine(sys_, s0)
    with eng(sys_, s0, mode) as g:
        g.step(120)
        c.step(120)
        ke, spg = g.read_kinetic()
        tot = g.read_kinetic_total()
        assert np.array_equal(g.read_positions(), c.state.pos)
        assert g.read_potential() == g.kicks()[1]
    st = c.state
    u = st.vel.astype(np.float64) * (1.0 / 4294967296.0) / sys_.dt
    want = 0.5 * np.array([1.0, 2.5])[st.species] * (u * u).sum(axis=1)
    assert np.array_equal(spg, st.species)
    assert np.allclose(ke, want, rtol=1e-14, atol=0.0)
    assert abs(tot - want.sum()) < 1e-12 * want.sum()


@pytest.mark.parametrize("mode", ["cells", "verlet"])
def test_observer_grid_matches_the_oracle(O, mode):
    """Observer::read (observe.rs:86-97) on a two-species fluid with species 1 pinned: the density
    grid of all particles and of species 0 equals the oracle's count for count, with grids that
    fit in shared memory and one that does not (200 x 100), taken between list builds (positions
    up to the skin outside the box); the kinetic energy equals the oracle's exact half-step sum.
    Mixing and segregation of the reading match the oracle's counts'. 3D engines refuse."""
    from micrographia_gb300 import Reading, mixing, segregation

    n = 3000
    sys_ = System(box_for(n, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0, 3.0])
    s0 = O.fluid(sys_, n, 1.0, 8)
    sp = (np.arange(n) % 4 == 0).astype(np.uint32)
    s0 = State(s0.pos, np.where(sp[:, None] == 1, 0, s0.vel).astype(np.int32), sp)
    sys_.with_pinned(1)
    m = ForceMode.cell_list() if mode == "cells" else ForceMode.verlet_with_skin(sys_, n, 0.5)
    with GpuEngine(sys_, s0, m) as g:
        for k, grid in enumerate([(16, 12), (1, 1), (200, 100), (33, 7)]):
            g.step(7)
            r = g.observe_grid(grid, 0)
            st = g.read_state()
            wa, wm = O.observer_grid(sys_, st, grid, 0)
            assert np.array_equal(r.all, wa)
            assert np.array_equal(r.marked, wm)
            assert r.kinetic == O.exact_kinetic(sys_, st)
            assert r.all.sum() == n and r.marked.sum() == (sp == 0).sum()
            want = Reading(wa, wm, 0.0)
            for f in (mixing, segregation):
                assert f(r) == f(want) or (math.isnan(f(r)) and math.isnan(f(want)))
    sys3 = System3(cube_for(500, 0.5), 0.005, Pair.wca(), [1.0])
    with GpuEngine3(sys3, O.fcc_maxwell(sys3, 500, 1.0, 1)) as g3:
        with pytest.raises(RuntimeError):
            _abi.check(g3._lib.gbmd_observe_grid(g3._h, 4, 4, 0, None, None, None))


def test_frame_between_list_builds(O):
    """Frames taken mid-way between list builds, when positions may sit outside [0, L) by up to
    the skin, count the same RDF and profile as the oracle on the wrapped state."""
    sys_, s = equilibrated(O, 3000, 0.7, Pair.lj(2.5), 4)
    with GpuEngine(sys_, s, ForceMode.verlet_with_skin(sys_, 3000, 0.5)) as g:
        for k in range(4):
            g.step(3)
            _, rdf, prof = g.observe(rdf_bins=128, rdf_rmax=4.0, profile_bins=50, profile_axis=1)
            st = g.read_state()
            assert np.array_equal(rdf, O.rdf(sys_, st, 128, 4.0))
            assert np.array_equal(prof, O.profile(sys_, st, 50, 1))


@pytest.mark.parametrize("dim", [2, 3])
def test_rdf_small_box_all_pairs(O, dim):
    """An RDF range wider than a third of the box counts every pair once (no cell list)."""
    if dim == 3:
        sys_, s = liquid3(O, 1000, 0.8, 1.0)
        eng = GpuEngine3
    else:
        sys_, s = equilibrated(O, 200, 0.7, Pair.lj(2.5), 4)
        eng = GpuEngine
    with eng(sys_, s) as g:
        g.step(5)
        _, rdf, _ = g.observe(rdf_bins=100, rdf_rmax=6.0)
        st = g.read_state()
    ref = O.rdf(sys_, st, 100, 6.0)
    assert np.array_equal(rdf, ref)
    assert ref.sum() > 0


@pytest.mark.parametrize("dim", [2, 3])
def test_rdf_and_profile_on_exact_bin_edges(O, dim):
    """A unit lattice in a box of whole sigmas: pair distances 1, 2, 3, 4 and 5 (= rmax) fall
    exactly on RDF bin edges and every particle exactly on a profile slab edge, so the f32
    estimates hand these to the f64 definition; the counts equal the oracle's."""
    side = 64 if dim == 2 else 16
    n = side**dim
    grid = np.stack(np.meshgrid(*[np.arange(side)] * dim, indexing="ij"), -1).reshape(n, dim)
    pos = (grid.astype(np.int64) * ONE).astype(np.int64)
    box = [side * ONE] * dim
    st = (State if dim == 2 else State3)(pos, np.zeros((n, dim), np.int32), np.zeros(n, np.uint32))
    if dim == 2:
        sys_, eng = System(box, 0.005, Pair.lj(2.5), [1.0]), GpuEngine
    else:
        sys_, eng = System3(box, 0.005, Pair.lj(2.5), [1.0]), GpuEngine3
    with eng(sys_, st, ForceMode.verlet_with_skin(sys_, n, 0.3)) as g:
        _, rdf, prof = g.observe(rdf_bins=200, rdf_rmax=5.0, profile_bins=side, profile_axis=dim - 1)
    want = O.rdf(sys_, st, 200, 5.0)
    assert np.array_equal(rdf, want)
    assert want[40] > 0 and want[80] > 0  # r = 1 and r = 2 exactly at the edges of bins 40, 80
    assert np.array_equal(prof, O.profile(sys_, st, side, dim - 1))
    assert np.all(prof == n // side)


def test_rdf_with_cells_wider_than_the_f32_offsets(O):
    """rmax = 45 sigma: RDF cells of ~47 sigma, beyond what the f32 cell offsets cover; the
    integer-separation kernel counts the same pairs as the oracle."""
    sys_, s = fluid(O, 1000, 0.05, Pair.lj(2.5), 8)
    with GpuEngine(sys_, s) as g:
        g.step(20)
        _, rdf, prof = g.observe(rdf_bins=100, rdf_rmax=45.0, profile_bins=10000, profile_axis=0)
        st = g.read_state()
    assert np.array_equal(rdf, O.rdf(sys_, st, 100, 45.0))
    assert np.array_equal(prof, O.profile(sys_, st, 10000, 0))  # more bins than shared memory holds


# ---------------------------------------------------------------- the Andersen heat bath
def _same_ledger(g, c):
    """The bath's ledger slot against the oracle's: redraws exactly, the energy exactly as the
    sum of the events rounded to 2^-24, and close to IntEngine's own f64 sum in particle order."""
    e, imp, h = g.read_ledger()
    oe, oef, oh, oclock = c.ledger()
    B = _abi.LEDGER_BATH
    assert h[B] == oh and oh > 0
    assert e[B] == oef / 2**24
    assert abs(e[B] - oe) <= oh * 2.0**-24 + 1e-12 * abs(oe) + 1e-9
    assert all(x == 0 for k, x in enumerate(h) if k != B) and not any(imp)
    return oclock


@pytest.mark.parametrize("mode,arith", [("verlet", _abi.ARITH_F32), ("cells", _abi.ARITH_F32), ("verlet", _abi.ARITH_INT)])
def test_bath_matches_oracle(O, mode, arith):
    """walls::andersen after the kick (int_engine.rs:275-293): the redraws, keyed on (id, clock),
    give the oracle's trajectory bit for bit across graph blocks, single steps and list rebuilds."""
    sys_, s0 = fluid(O, 3000, 0.6, Pair.lj(2.5), 21, t=2.0)
    sys_.with_thermostat(0.8, 4.0)
    m = ForceMode.verlet_with_skin(sys_, 3000, 0.3) if mode == "verlet" else ForceMode.cell_list()
    c = O.IntEngine(sys_, s0, integer=arith == _abi.ARITH_INT)
    with GpuEngine(sys_, s0, m, arith=arith) as g:
        for k in (37, 100, 1, 63):
            g.step(k)
            c.step(k)
            assert g.read_state() == c.state, k
        clock = _same_ledger(g, c)
        assert clock == 201


def test_bath_fan_and_layer_match_oracle(O):
    """with_fan (species mask, an x range, a drift) and with_bath_layer (a y range), with two
    species of different mass and a third pinned species the bath must skip."""
    n = 4000
    sys_ = System(box_for(n, 0.55, 1.0), 0.005, Pair.lj(2.5), [1.0, 2.0, 1.0]).with_pinned(2)
    L = sys_.box_f64()
    st = O.fluid(sys_, n, 1.2, 22)
    rng = np.random.default_rng(22)
    st.species[:] = rng.integers(0, 3, n).astype(np.uint32)
    st.vel[st.species == 2] = 0
    for build in (lambda s: s.with_thermostat(1.5, 6.0).with_fan(0b011, 0.2 * L[0], 0.6 * L[0], 0.7),
                  lambda s: s.with_thermostat(0.5, 6.0).with_bath_layer(0.1 * L[1], 0.5 * L[1])):
        import copy

        sb = build(copy.deepcopy(sys_))
        c = O.IntEngine(sb, st)
        with GpuEngine(sb, st, ForceMode.verlet_with_skin(sb, n, 0.3)) as g:
            for k in (50, 120):
                g.step(k)
                c.step(k)
                assert g.read_state() == c.state
            _same_ledger(g, c)
            assert np.array_equal(g.read_state().pos[st.species == 2], st.pos[st.species == 2])


def test_bath_3d_matches_oracle(O):
    """three::andersen (three.rs:247-265): three components, the species mask."""
    sys3, s0 = liquid3(O, 4000, 0.8442, 0.5)
    sys3.masses = [1.0, 3.0]
    sys3.pairs = sys3.pairs * 4
    s0.species[::3] = 1
    sys3.with_thermostat(1.2, 5.0)
    sys3.thermostat.species = 0b10
    c = O.IntEngine(sys3, s0)
    with GpuEngine3(sys3, s0, ForceMode.verlet_with_skin(sys3, 4000, 0.3)) as g:
        for k in (64, 27):
            g.step(k)
            c.step(k)
            assert g.read_state() == c.state
        _same_ledger(g, c)


def test_bath_added_at_run_time_and_resumed_from_a_snapshot(O):
    """update_system adds the bath mid-run (the clock counts every step since creation); a
    snapshot taken later resumes in a fresh engine with the same clock and the same draws."""
    import copy

    sys_, s0 = fluid(O, 3000, 0.6, Pair.lj(2.5), 23, t=1.5)
    c = O.IntEngine(sys_, s0)
    hot = copy.deepcopy(sys_).with_thermostat(0.6, 5.0)
    with GpuEngine(sys_, s0, ForceMode.verlet_with_skin(sys_, 3000, 0.3)) as g:
        g.step(40)
        c.step(40)
        g.update_system(hot)
        c.update_system(hot)
        g.step(70)
        c.step(70)
        assert g.read_state() == c.state
        snap = g.snapshot()
    with GpuEngine(hot, s0, ForceMode.verlet_with_skin(hot, 3000, 0.3)) as h:
        h.restore(snap)
        h.step(90)
        c.step(90)
        assert h.read_state() == c.state


def test_bath_thermalises():
    """md/tests/boundaries.rs:189-202: from T = 2, a bath at T = 0.8 (rate 1) holds the
    half-step temperature within 0.04 of 0.8 over steps 3000-5000."""
    n = 5000
    sys_ = System(box_for(n, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0]).with_thermostat(0.8, 1.0)
    s0 = init_state(sys_, _abi.INIT_FLUID, n, 2.0, 12, 0.1)
    with GpuEngine(sys_, s0) as g:
        g.step(3000)
        t = 0.0
        for _ in range(20):
            g.step(100)
            st = g.read_state()
            v = st.vel.astype(np.float64) / 2**32 / sys_.dt
            t += 0.5 * (v * v).sum() / n / 20
    assert abs(t - 0.8) < 0.04, t


def test_batch_bath_matches_each_plain_run(O):
    """Baths in a batch: systems with and without one, each equal to its own IntEngine run
    (ids counted from the system's first particle, the batch's clock), each with its own ledger."""
    from micrographia_gb300 import BatchEngine, workloads

    cfg = workloads.config4(count=6, base_seed=31, n_min=600, n_max=3000)
    systems = [s for s, _ in cfg]
    for k, sys_ in enumerate(systems):
        if k % 3 != 1:
            sys_.with_thermostat(0.6 + 0.2 * k, 3.0 + k)
        if k == 2:
            L = sys_.box_f64()
            sys_.with_fan(0b1, 0.1 * L[0], 0.7 * L[0], 0.4)
    states = [O.init(s, spec) for s, spec in cfg]
    with BatchEngine(systems, states, ForceMode.verlet_with_skin(None, 0, 0.3)) as b:
        b.step(130)
        for k, (sys_, st) in enumerate(zip(systems, states)):
            c = O.IntEngine(sys_, st)
            c.step(130)
            assert b.read_system(k) == c.state, k
            e, _, h = b.read_ledger(k)
            oe, oef, oh, _ = c.ledger()
            assert h[_abi.LEDGER_BATH] == oh and e[_abi.LEDGER_BATH] == oef / 2**24, k
            assert (oh > 0) == (sys_.thermostat is not None)


# ---------------------------------------------------------------- checkpoint / resume
@pytest.mark.parametrize("dim", [2, 3])
def test_snapshot_resume_is_bit_identical(O, dim):
    """2N steps against N steps, snapshot, restore into another engine, N steps: the same state
    bit for bit (2D with the rescale thermostat, whose phase the snapshot carries); a snapshot
    with one flipped bit is refused."""
    from micrographia_gb300 import snapshot

    if dim == 2:
        n = 4000
        sys_ = System(box_for(n, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0])
        s0 = O.fluid(sys_, n, 1.0, 5)
        kw, eng = dict(rescale_every=10, rescale_t=0.8), GpuEngine
    else:
        sys_, s0 = liquid3(O, 4000, 0.8, 1.0)
        kw, eng = {}, GpuEngine3
    with eng(sys_, s0, **kw) as a:
        a.step(137)
        a.step(140)
        want = a.read_state()
    with eng(sys_, s0, **kw) as b:
        b.step(137)
        snap = b.snapshot()
        st = b.read_state()
    d, pos, vel, sp, steps, clock, phase = snapshot.unpack(snap)
    assert (d, steps, phase) == (dim, 137, 137)
    assert np.array_equal(pos, st.pos.reshape(-1, dim)) and np.array_equal(vel, st.vel.reshape(-1, dim))
    with eng(sys_, s0, **kw) as c:
        c.step(11)
        c.restore(snap)
        c.step(140)
        assert c.read_state() == want
        bad = bytearray(snap)
        bad[-5] ^= 1
        with pytest.raises(_abi.GbmdError):
            c.restore(bytes(bad))


# ---------------------------------------------------------------- all-integer table forces (md-core table.rs)
def golden_int_setup(O):
    """md/src/checks.rs:155-167: 3000-particle binary LJ mixture, rho 0.6, seed 2026."""
    sys_ = System(box_for(3000, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0, 2.0]).with_pair(0, 1, Pair(0.7, 1.05, 2.5))
    s = O.fluid(sys_, 3000, 1.0, 2026)
    s.species[::4] = 1
    s.vel = O.maxwell(sys_, s.species, 1.0, 2026)
    return sys_, s


@pytest.mark.parametrize("mode", ["cells", "verlet"])
def test_golden_int_hash_on_gpu(O, mode):
    """The reference's own golden vector, reproduced on the GPU: GOLDEN_INT_HASH after 1000
    all-integer steps (md/tests/integer.rs:84-98)."""
    import json
    import os

    golden = int(json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.json")))["golden_int_hash"], 16)
    sys_, s = golden_int_setup(O)
    m = ForceMode.cell_list() if mode == "cells" else ForceMode.verlet_for(sys_, 3000)
    with GpuEngine(sys_, s, m, arith=_abi.ARITH_INT) as g:
        g.step(1000)
        assert g.read_state().hash() == golden


def test_integer_kicks_match_oracle_2d_and_3d(O):
    sys_, s = golden_int_setup(O)
    cpu = O.IntEngine(sys_, s, f64=True, integer=True)
    cpu.step(50)
    st = cpu.state
    for m in (ForceMode.cell_list(), ForceMode.verlet_for(sys_, 3000)):
        with GpuEngine(sys_, st, m, arith=_abi.ARITH_INT) as g:
            kg, pe = g.kicks()
        kc, pec = cpu.kicks()
        assert np.array_equal(kg, kc)
        assert abs(pe - pec) < 1e-10 * abs(pec)  # f64 pair energies summed in another order
    sys3, s3 = liquid3(O, 4000, 0.8, 1.0)
    c3 = O.IntEngine(sys3, s3, f64=True, integer=True)
    c3.step(20)
    st3 = c3.state
    with GpuEngine3(sys3, st3, arith=_abi.ARITH_INT) as g:
        g.step(15)
        c3.step(15)
        assert g.read_state() == c3.state
        kg, _ = g.kicks()
        assert np.array_equal(kg, c3.kicks()[0])
        # whole 64-step graph blocks (a small single-species engine): still the integer tables
        g.step(130)
        c3.step(130)
        assert g.read_state() == c3.state


# ---------------------------------------------------------------- FP64 reference kicks (IntEngine<f64>)
@pytest.mark.parametrize("mode", ["cells", "verlet"])
def test_f64_kicks_match_oracle_2d(O, mode):
    sys_ = System(box_for(3000, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0, 3.0]).with_pair(0, 1, Pair(0.6, 1.1, 2.5))
    s = O.fluid(sys_, 3000, 1.0, 1)
    s.species[::3] = 1
    s.vel = O.maxwell(sys_, s.species, 1.0, 1)
    cpu = O.IntEngine(sys_, s)
    cpu.step(60)
    st = cpu.state
    m = ForceMode.cell_list() if mode == "cells" else ForceMode.verlet_for(sys_, 3000)
    with GpuEngine(sys_, st, m) as g:
        k64, pe64 = g.kicks_f64()
        k32, _ = g.kicks()
    want, want_pe = O.IntEngine(sys_, st, f64=True).kicks()
    assert np.array_equal(k64, want)
    assert abs(pe64 - want_pe) < 1e-12 * abs(want_pe)  # f64 sums in another order
    rel = math.sqrt(((k32.astype(np.float64) - k64) ** 2).sum() / (k64.astype(np.float64) ** 2).sum())
    assert rel < 1e-5  # md-ref physics.rs:144


def test_f64_kicks_match_oracle_3d(O):
    sys3, s = liquid3(O, 4000, 0.8, 1.0)
    cpu = O.IntEngine(sys3, s)
    cpu.step(30)
    st = cpu.state
    with GpuEngine3(sys3, st) as g:
        g.step(7)  # positions unwrapped between list builds
        st = g.read_state()
        k64, _ = g.kicks_f64()
    want, _ = O.IntEngine(sys3, st, f64=True).kicks()
    assert np.array_equal(k64, want)


# ---------------------------------------------------------------- the pair arithmetic's own reciprocal and division
@pytest.mark.parametrize(
    "pairs",
    [
        [Pair.lj(2.5)],
        [Pair.wca()],
        [Pair.lj(2.5), Pair(0.6, 1.1, 2.5), Pair(0.6, 1.1, 2.5), Pair(0.3, 0.8, 3.0)],
    ],
    ids=["lj", "wca", "mixture"],
)
def test_pair_math_matches_library(pairs):
    """rcp_cr / div_cr equal __frcp_rn / __fdiv_rn bit for bit: every f32 of [2^50, 2^63), every
    scaled r2 of each pair type's fast range through the LJ chain, and 2^28 random quotients."""
    import ctypes as C

    ns = 1 if len(pairs) == 1 else 2
    sys_ = System(box_for(1000, 0.7, 1.0), 0.005, pairs[0], [1.0] * ns)
    if ns == 2:
        sys_ = sys_.with_pair(0, 1, pairs[1]).with_pair(1, 1, pairs[3])
    checked, bad = C.c_uint64(), C.c_uint64()
    cs = sys_.to_c()
    _abi.check(_abi.lib().gbmd_check_pair_math(C.byref(cs), 1 << 28, 0, C.byref(checked), C.byref(bad)))
    assert bad.value == 0
    assert checked.value > (13 << 23) + (1 << 28)


# ---------------------------------------------------------------- velocity-rescale thermostat (the 2D slab workload)
def test_rescale_thermostat_matches_oracle(O):
    """Slab start, rescale to T = 0.45 every 10 steps: the GPU trajectory equals the oracle's
    (IntEngine<f32> stepped one step at a time, the exact-integer rescale after every 10th)."""
    n = 20000
    sys_ = System(box_for(n, 0.2125, 4.0), 0.005, Pair.lj(2.5), [1.0])
    s0 = O.init(sys_, make_init(_abi.INIT_SLAB, n, 0.45, 7, 0.1, 0.7, 0.05, 0.25))
    with GpuEngine(sys_, s0, ForceMode.verlet_with_skin(sys_, n, 0.3), rescale_every=10, rescale_t=0.45) as g:
        c = O.IntEngine(sys_, s0)
        g.step(7)
        g.step(88)  # crosses a 60-step graph block and single steps either side
        for k in range(95):
            c.step(1)
            if (k + 1) % 10 == 0:
                st = c.state
                st.vel = O.set_temperature(sys_, st, 0.45, exact=True)
                c.set_state(st)
        got = g.read_state()
        assert got == c.state
        assert got.velocity_sum() == [0, 0]


# ---------------------------------------------------------------- full size (configs 2): size-independent properties
def test_config2_full_size_properties(O):
    """3D FCC N=1,048,576, rho 0.8442, T 0.72, skin 0.3: momentum stays exactly zero, the run
    reverses bit for bit, and the lists never overflow."""
    n = 1 << 20
    sys3 = System3(cube_for(n, 0.8442), 0.005, Pair.lj(2.5), [1.0])
    spec = make_init(_abi.INIT_FCC, n, 0.72, 1, 0.05)
    with GpuEngine3(sys3, None, ForceMode.verlet_with_skin(sys3, n, 0.3), init=spec) as g:
        s0 = g.read_state()
        g.step(100)
        s1 = g.read_state()
        assert s1.velocity_sum() == [0, 0, 0]
        rebuilds, overflow = g.read_list_stats()
        assert not overflow and rebuilds >= 2
        g.reverse()
        g.step(100)
        g.reverse()
        assert g.read_state().hash() == s0.hash()


def test_slab_full_size_properties():
    """2D liquid-vapour slab, N = 2^24 (4:1 box, liquid 0.70, vapour 0.05), skin 0.3, NVE: the
    velocity sum stays exactly zero, the lists never overflow, and 60 steps reverse bit for bit
    (the state hash of the initial state is recovered)."""
    from micrographia_gb300 import workloads

    sys_, spec = workloads.config3(1 << 24)
    n = spec.n
    with GpuEngine(sys_, None, ForceMode.verlet_with_skin(sys_, n, 0.3), init=spec) as g:
        h0 = g.state_hash()
        g.step(60)
        assert g.read_state().velocity_sum() == [0, 0]
        rebuilds, overflow = g.read_list_stats()
        assert not overflow and rebuilds >= 1
        g.reverse()
        g.step(60)
        g.reverse()
        assert g.state_hash() == h0


# ---------------------------------------------------------------- batched replicas
def test_batch_replicas_match_their_plain_runs(O):
    """Uneven 2D systems stepped in one batch: each replica's state equals md-ref's IntEngine<f32>
    run of that system alone, bit for bit (through a 100-step graph block and single steps)."""
    from micrographia_gb300 import BatchEngine, workloads

    cfg = workloads.config4(count=10, base_seed=5, n_min=256, n_max=4096)
    systems = [s for s, _ in cfg]
    states = [O.init(s, spec) for s, spec in cfg]
    with BatchEngine(systems, states, ForceMode.verlet_with_skin(None, 0, 0.3)) as b:
        b.step(150)
        launches, rebuilds = b.stats()
        assert rebuilds >= 2
        for k, (sys_, st) in enumerate(zip(systems, states)):
            c = O.IntEngine(sys_, st)
            c.step(150)
            assert b.read_system(k) == c.state, k


def test_batch_skin_tuner_keeps_the_trajectory(O):
    """The autotuner picks a skin and a force-lane split from timed trial runs on the given states;
    the replicas still equal their plain oracle runs bit for bit at that choice, and at every
    force-lane split asked for."""
    from micrographia_gb300 import BatchEngine, workloads

    cfg = workloads.config4(count=6, base_seed=9, n_min=512, n_max=4096)
    systems = [s for s, _ in cfg]
    states = [O.init(s, spec) for s, spec in cfg]
    with BatchEngine(systems, states, ForceMode.verlet_with_skin(None, 0, 0.3), tune_skin=True) as b:
        assert b.skin in (0.3, 0.4, 0.5, 0.6, 0.7)
        assert b.force_lanes in (1, 2, 4)
        b.step(120)
        for k, (sys_, st) in enumerate(zip(systems, states)):
            c = O.IntEngine(sys_, st)
            c.step(120)
            assert b.read_system(k) == c.state, k
    with BatchEngine(systems, states, ForceMode.verlet_with_skin(None, 0, 0.45)) as b:
        assert b.skin == 0.45
        assert b.force_lanes == 1
    for lanes in (2, 4):  # every force-lane split gives the same trajectory
        with BatchEngine(systems, states, ForceMode.verlet_with_skin(None, 0, 0.3), force_lanes=lanes) as b:
            assert b.force_lanes == lanes
            b.step(120)
            for k, (sys_, st) in enumerate(zip(systems, states)):
                c = O.IntEngine(sys_, st)
                c.step(120)
                assert b.read_system(k) == c.state, (lanes, k)


def test_batch_3d(O):
    from micrographia_gb300 import BatchEngine

    systems, states = [], []
    for k, (n, rho) in enumerate([(500, 0.8), (2048, 0.6), (864, 0.85)]):
        s3 = System3(cube_for(n, rho), 0.005, Pair.lj(2.5), [1.0])
        systems.append(s3)
        states.append(O.fcc_maxwell(s3, n, 0.9, 10 + k))
    with BatchEngine(systems, states, ForceMode.verlet_with_skin(None, 0, 0.3)) as b:
        b.step(60)
        for k in range(3):
            c = O.IntEngine(systems[k], states[k])
            c.step(60)
            assert b.read_system(k) == c.state


@pytest.mark.parametrize("dim", [2, 3])
def test_batch_frames_equal_plain_frames(O, dim):
    """gbmd_batch_observe: every system's frame of a batch (uneven sizes, small boxes where the RDF
    range covers the whole box included) equals a plain engine's frame of that system at the same
    step: RDF counts exactly, kinetic and potential energy, virial, temperature and pressure to
    1e-12 relative (the same terms summed in another order); the states stay bit-identical."""
    from micrographia_gb300 import BatchEngine

    if dim == 2:
        sizes = [(300, 0.5), (1500, 0.8), (4000, 0.35), (700, 0.7)]
        systems = [System(box_for(n, rho, 1.0), 0.005, Pair.lj(2.5), [1.0]).with_seed(40 + k) for k, (n, rho) in enumerate(sizes)]
        states = [O.fluid(s, n, 1.1, 40 + k) for k, (s, (n, _)) in enumerate(zip(systems, sizes))]
    else:
        sizes = [(500, 0.8), (2048, 0.6), (864, 0.85)]
        systems = [System3(cube_for(n, rho), 0.005, Pair.lj(2.5), [1.0]) for n, rho in sizes]
        states = [O.fcc_maxwell(s, n, 0.9, 50 + k) for k, (s, (n, _)) in enumerate(zip(systems, sizes))]
    bins, rmax = 64, 4.0
    with BatchEngine(systems, states, ForceMode.verlet_with_skin(None, 0, 0.3), block_steps=50) as b:
        for steps in (0, 137, 100):
            b.step(steps)
            frames, rdf = b.observe(rdf_bins=bins, rdf_rmax=rmax)
            got = b.read_all()
            for k, (sys_, st) in enumerate(zip(systems, states)):
                cls = GpuEngine if dim == 2 else GpuEngine3
                with cls(sys_, got[k], ForceMode.verlet_with_skin(sys_, st.n(), 0.3)) as g:
                    f, r, _ = g.observe(rdf_bins=bins, rdf_rmax=rmax)
                assert np.array_equal(rdf[k], r), (steps, k)
                for name in ("kinetic", "potential", "virial", "temperature", "pressure"):
                    x, y = getattr(frames[k], name), getattr(f, name)
                    assert abs(x - y) <= 1e-12 * max(abs(y), 1.0), (steps, k, name, x, y)
                assert frames[k].n == f.n and frames[k].volume == f.volume
        # the batch's states still follow the oracle
        for k, (sys_, st) in enumerate(zip(systems, states)):
            c = O.IntEngine(sys_, st)
            c.step(237)
            assert got[k] == c.state, k


# ---------------------------------------------------------------- serving
def _drain(sv, want_last, limit_s=120.0):
    import time

    frames, last = [], {}
    t0 = time.time()
    while len(last) < want_last:
        for f in sv.poll():
            frames.append(f)
            if f.last:
                last[f.request] = f
        if time.time() - t0 > limit_s:
            raise AssertionError("serving loop did not finish in time")
        time.sleep(0.001)
    return frames, last


@pytest.mark.parametrize("lanes", [True, False])
def test_served_results_equal_solo_runs(O, lanes):
    """Mixed 2D/3D requests, more than the server holds at once, served in lanes (stepped together
    in batches that members join and leave at frame boundaries) or each on its own engine: each
    request's final state is bit-identical to the same request run alone and to the oracle's
    IntEngine run; its RDF counts equal the solo run's exactly and its energies and virial agree
    to 1e-12 relative (a lane sums the same terms in another order; an engine bit for bit)."""
    from micrographia_gb300 import Server, workloads

    cfg = workloads.config5(count=8, rate=1e9, base_seed=3, n_min=800, n_max=6000)
    with Server(hbm_budget_bytes=4 << 30, max_active=3, lane_max_n=None if lanes else 0) as sv:
        ids = [sv.submit(s, spec, steps=300, frame_every=100, rdf_bins=64, rdf_rmax=4.0) for _, s, spec in cfg]
        frames, last = _drain(sv, len(ids))
        st = sv.stats()
    if lanes:
        assert st.lane_requests == len(ids)
        assert st.lane_repacks >= 3  # members joined and left at frame boundaries
    else:
        assert st.lane_requests == 0
    by_req = {}
    for f in frames:
        by_req.setdefault(f.request, []).append(f)
    for rid, (_, s, spec) in zip(ids, cfg):
        cls = GpuEngine if s.DIM == 2 else GpuEngine3
        with cls(s, None, ForceMode.verlet_with_skin(s, spec.n, 0.3), init=spec, block_steps=100) as g:
            solo = []
            for _ in range(3):
                g.step(100)
                f, rdf, _ = g.observe(rdf_bins=64, rdf_rmax=4.0)
                solo.append((f.kinetic, f.potential, f.virial, list(rdf)))
            h = g.state_hash()
        served = [(f.frame.kinetic, f.frame.potential, f.frame.virial, list(f.rdf[:64])) for f in sorted(by_req[rid], key=lambda f: f.index)]
        assert len(served) == 3
        for (k1, p1, w1, r1), (k2, p2, w2, r2) in zip(served, solo):
            assert r1 == r2
            if lanes:
                for x, y in ((k1, k2), (p1, p2), (w1, w2)):
                    assert abs(x - y) <= 1e-12 * max(abs(y), 1.0)
            else:
                assert (k1, p1, w1) == (k2, p2, w2)
        assert [f.frame.step for f in sorted(by_req[rid], key=lambda f: f.index)] == [100, 200, 300]
        assert last[rid].state_hash == h
        c = O.IntEngine(s, O.init(s, spec))
        c.step(300)
        assert h == c.hash()


def test_served_lanes_and_engines_mix():
    """Requests routed both ways at once: small ones with the lane's cadence into lanes, a large one
    and one with another frame cadence onto engines; a request cancelled while in a lane leaves it
    at the next frame boundary with its last frame; every other request finishes with the final
    state of its solo run."""
    from micrographia_gb300 import Server, workloads

    cfg = workloads.config5(count=6, rate=1e9, base_seed=21, n_min=600, n_max=5000)
    with Server(hbm_budget_bytes=4 << 30, max_active=8, lane_max_n=3000) as sv:
        ids = []
        for k, (_, s, spec) in enumerate(cfg):
            every = 50 if k == 5 else 100  # (the 3D lane has taken a cadence of 100 by then)
            ids.append(sv.submit(s, spec, steps=400, frame_every=every, rdf_bins=32, rdf_rmax=3.0))
        sv.poll()
        small = [rid for rid, (_, s, spec) in zip(ids, cfg) if spec.n <= 3000 and rid != ids[5]]
        victim = small[-1]
        sv.cancel(victim)
        frames, last = _drain(sv, len(ids))
        st = sv.stats()
    assert st.lane_requests == len(small)
    assert st.completed == len(ids)
    by_req = {}
    for f in frames:
        by_req.setdefault(f.request, []).append(f)
    assert len(by_req[ids[5]]) == 8  # its own cadence, on an engine
    assert len(by_req[victim]) < 4
    for rid, (_, s, spec) in zip(ids, cfg):
        if rid == victim:
            continue
        cls = GpuEngine if s.DIM == 2 else GpuEngine3
        with cls(s, None, ForceMode.verlet_with_skin(s, spec.n, 0.3), init=spec) as g:
            g.step(400)
            assert last[rid].state_hash == g.state_hash()


def test_served_bath_requests_equal_the_oracle(O):
    """Requests whose systems carry a heat bath: the served final state equals IntEngine's run
    of the same system (the bath keyed on each request's own ids and step clock)."""
    from micrographia_gb300 import Server, workloads

    cfg = workloads.config5(count=4, rate=1e9, base_seed=17, n_min=800, n_max=3000)
    for k, (_, s, _) in enumerate(cfg):
        s.with_thermostat(0.7 + 0.3 * k, 2.0 + k)
    with Server(hbm_budget_bytes=4 << 30, max_active=2) as sv:
        ids = [sv.submit(s, spec, steps=200, frame_every=100, rdf_bins=0) for _, s, spec in cfg]
        _, last = _drain(sv, len(ids))
    for rid, (_, s, spec) in zip(ids, cfg):
        c = O.IntEngine(s, O.init(s, spec))
        c.step(200)
        assert last[rid].state_hash == c.hash()
        assert c.ledger()[2] > 0


def test_server_budget_and_cancel():
    from micrographia_gb300 import Server, _abi, workloads

    cfg = workloads.config5(count=3, rate=1e9, base_seed=9, n_min=1024, n_max=2048)
    need = max(_abi.lib().gbmd_serve_estimate_bytes(__import__("ctypes").byref(s.to_c()), spec.n, 0.3) for _, s, spec in cfg)
    # room for one request at a time: the others wait and are admitted as memory frees up
    with Server(hbm_budget_bytes=need + need // 2, max_active=8) as sv:
        ids = [sv.submit(s, spec, steps=200, frame_every=100, rdf_bins=0) for _, s, spec in cfg]
        sv.poll()
        assert sv.stats().active == 1
        sv.cancel(ids[2])
        frames, last = _drain(sv, 2)
        assert set(last) == set(ids[:2])
        assert sv.stats().completed == 2
    # a request larger than the whole budget is refused with a budget error
    with Server(hbm_budget_bytes=1 << 20) as sv:
        _, s, spec = cfg[0]
        sv.submit(s, spec, steps=10)
        with pytest.raises(_abi.GbmdError) as ei:
            sv.poll()
        assert ei.value.code == _abi.E_BUDGET


def test_step_loop_barrier_runs_out_with_a_status(O):
    """The grid barrier's bounded wait: a cooperative launch whose block 0 never arrives makes the
    other blocks give up; the engine reports GBMD_E_TIMEOUT and refuses further steps, and the
    GPU stays usable (a new engine steps normally afterwards)."""
    sys3, s0 = liquid3(O, 4000, 0.8442, 0.72)
    with GpuEngine3(sys3, s0) as g:
        assert g.debug_barrier_timeout(4) == _abi.E_TIMEOUT
        assert b"ran out of time" in _abi.lib().gbmd_last_error()
        with pytest.raises(RuntimeError):
            g.step(1)
    with GpuEngine3(sys3, s0) as g:
        c = O.IntEngine(sys3, s0)
        g.step(70)
        c.step(70)
        assert g.read_state() == c.state


@pytest.mark.parametrize("n,loop", [(4000, True), (4000, False), (120_000, False)])
def test_list_overflow_is_reported(O, n, loop):
    """A list capacity below the neighbour count: the build clamps the lists and sets the
    overflow word; the engine reports GBMD_E_OVERFLOW and refuses further steps, in the step loop
    and in per-step graphs alike; an upload clears the failed state."""
    sys3, s0 = liquid3(O, n, 0.8442, 0.72)
    flags = 0 if loop else _abi.FLAG_NO_STEP_LOOP
    with GpuEngine3(sys3, s0, ForceMode.verlet_with_skin(sys3, n, 0.3, cap=16), flags=flags) as g:
        g.step(70)
        with pytest.raises(_abi.GbmdError) as err:
            g.wait()
        assert err.value.code == _abi.E_OVERFLOW
        assert g.read_list_stats()[1]
        with pytest.raises(_abi.GbmdError):
            g.step(1)
        g.upload(s0)
        assert g.read_state() == s0


# ---------------------------------------------------------------- page commands (engine.rs:895-1063)
@pytest.mark.parametrize("dim", [2, 3])
def test_kick_region_and_species_velocity_match_oracle(O, dim):
    """kick_region (md.wgsl:216-229, md3.wgsl:541-553) and set_species_velocity against their
    restatements, then the trajectory after them against IntEngine (through 64-step blocks)."""
    if dim == 3:
        sys_, s0 = liquid3(O, 4000, 0.8442, 0.9)
        eng = GpuEngine3
    else:
        sys_, s0 = fluid(O, 6000, 0.7, Pair.lj(2.5), 4)
        eng = GpuEngine
    L = [b / 2**32 for b in sys_.box_len]
    lo, hi = [0.2 * x for x in L], [0.65 * x for x in L]
    with eng(sys_, s0, ForceMode.verlet_with_skin(sys_, s0.n(), 0.3)) as g:
        g.step(70)
        st = g.read_state()
        g.kick_region(lo, hi, 1.37, [0.25, -0.5, 0.125][:dim])
        want = O.kick_region(sys_, st, lo, hi, 1.37, [0.25, -0.5, 0.125][:dim])
        got = g.read_state()
        assert got == want
        assert (got.vel != st.vel).any(axis=1).sum() > s0.n() // 20
        g.kick_region([0.0] * dim, [1.01 * x for x in L], 0.0, [0.0] * dim)  # freeze everything
        frozen = g.read_state()
        assert not frozen.vel.any()
        g.set_species_velocity(0, [0.5, 0.25, -0.125][:dim])
        got = g.read_state()
        assert got == O.set_species_velocity(sys_, frozen, 0, [0.5, 0.25, -0.125][:dim])
        assert np.array_equal(got.vel[0], [O.to_step_displacement(sys_, v) for v in [0.5, 0.25, -0.125][:dim]])
        c = O.IntEngine(sys_, got)
        g.step(140)
        c.step(140)
        assert g.read_state() == c.state


def test_set_species_and_sort_now_match_oracle(O):
    """set_species on a binary mixture (masses and pair constants follow the new species), a
    forced re-sort, and the trajectory after both against IntEngine."""
    sys_ = System(box_for(4000, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0, 3.0]).with_pair(0, 1, Pair(0.6, 1.1, 2.5))
    s = O.fluid(sys_, 4000, 1.0, 3)
    s.species[::4] = 1
    s.vel = O.maxwell(sys_, s.species, 1.0, 3)
    with GpuEngine(sys_, s, ForceMode.verlet_with_skin(sys_, 4000, 0.3)) as g:
        g.step(50)
        st = g.read_state()
        ids = np.arange(0, 4000, 7, dtype=np.uint32)
        g.set_species(np.concatenate([ids, ids[:10]]), 1)
        want = O.set_species(st, ids, 1)
        assert g.read_state() == want
        g.sort_now()
        assert g.read_state() == want
        c = O.IntEngine(sys_, want)
        g.step(100)
        c.step(100)
        assert g.read_state() == c.state
        with pytest.raises(_abi.GbmdError):
            g.set_species([1], 2)  # no species 2


@pytest.mark.parametrize("dim", [2, 3])
def test_update_system_matches_oracle(O, dim):
    """update_system (engine.rs:895-934): new pair constants (a smaller cutoff), masses, gravity and
    dt from the next step; the trajectory equals IntEngine run on the new system from that state.
    A cutoff above the engine's largest, or another box, is refused with the engine unchanged."""
    import copy

    if dim == 3:
        sys_, s0 = liquid3(O, 4000, 0.8442, 0.9)
        eng = GpuEngine3
    else:
        sys_, s0 = fluid(O, 6000, 0.7, Pair.lj(2.5), 6)
        eng = GpuEngine
    with eng(sys_, s0, ForceMode.verlet_with_skin(sys_, s0.n(), 0.3)) as g:
        g.step(70)
        st = g.read_state()
        new = copy.deepcopy(sys_)
        new.pairs = [Pair(1.3, 1.0, 2.2) for _ in new.pairs]
        new.masses = [1.7]
        new.dt = 0.004
        new.gravity = [0.0, -0.3, 0.0][:dim]
        g.update_system(new)
        c = O.IntEngine(new, st)
        g.step(150)
        c.step(150)
        assert g.read_state() == c.state
        bad = copy.deepcopy(new)
        bad.pairs = [Pair(1.0, 1.0, 2.9) for _ in bad.pairs]
        with pytest.raises(_abi.GbmdError):
            g.update_system(bad)
        g.step(10)
        c.step(10)
        assert g.read_state() == c.state


# ---------------------------------------------------------------- direct-launch timing paths
def test_time_loop_and_batch_time_phases_keep_the_trajectory(O):
    """The timing entry points step with direct launches (the persistent loop; the batch's force
    and rebuild kernels) instead of graphs: the trajectories still equal the oracle's."""
    from micrographia_gb300 import BatchEngine, workloads

    sys3, st = liquid3(O, 8000, 0.8442, 1.0)
    with GpuEngine3(sys3, st, ForceMode.verlet_with_skin(sys3, 8000, 0.3)) as g:
        taken, ms, launches = g.time_loop(100)
        assert taken >= 100 and launches >= 1 and ms > 0
        got = g.read_state()
    cpu = O.IntEngine(sys3, st)
    cpu.step(taken)
    assert got == cpu.state
    cfg = workloads.config4(count=6, base_seed=3, n_min=256, n_max=4096)
    systems = [s for s, _ in cfg]
    states = [O.init(s, spec) for s, spec in cfg]
    with BatchEngine(systems, states, ForceMode.verlet_with_skin(None, 0, 0.3)) as b:
        b.step(30)
        f, r, nr = b.time_phases(70)
        assert f > 0 and nr >= 1
        for k, (sys_, s0) in enumerate(zip(systems, states)):
            c = O.IntEngine(sys_, s0)
            c.step(100)
            assert b.read_system(k) == c.state, k


def test_flip_species_bit_matches_the_oracle(O):
    """GpuEngine::flip_species_bit (engine.rs:1014-1024): bit 30 of x of every particle of species 1
    flipped between steps; the run then equals the oracle's from the same flipped state."""
    n = 3000
    sys_ = System(box_for(n, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0, 2.0])
    s0 = O.fluid(sys_, n, 1.0, 61)
    s0.species[:] = np.arange(n) % 2
    c = O.IntEngine(sys_, s0)
    with GpuEngine(sys_, s0, ForceMode.verlet_with_skin(sys_, n, 0.3)) as g:
        g.step(200)
        c.step(200)
        st = c.state.copy()
        st.pos[st.species == 1, 0] ^= np.int64(1 << 30)
        g.flip_species_bit(0b10, 0, 30)
        c2 = O.IntEngine(sys_, st)
        g.step(200)
        c2.step(200)
        assert g.read_state() == c2.state
