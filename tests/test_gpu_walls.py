"""Walls on the GPU engine (md_core::walls, walls.rs): hard, soft and thermal walls, against the
oracle's IntEngine (md-ref int_engine.rs:203-227, 256-263, 316-330, 363-390; int_engine3.rs:107-126,
140-145, 186-205), bit for bit, with the ledger.

The ledger is compared exactly in the order-free form the engine keeps (each event's energy change
and impulse rounded to 2^-24 and summed as integers; the hit counts), and the oracle's f64 sums in
particle order within half a unit of 2^-24 per event. The scenarios follow the reference's own wall
tests (crates/md-ref/tests/boundaries.rs:6-110)."""

import numpy as np
import pytest

from micrographia_gb300 import ONE, ForceMode, GpuEngine, GpuEngine3, Pair, State, State3, System, System3, Wall, box_for, cube_for

pytestmark = pytest.mark.gpu


def _same_ledger(g, c):
    """GPU ledger (each event rounded to 2^-24, integer sums) against the oracle's."""
    ge, gp, gh = g.read_ledger()
    oe, op = c.wall_ledger_fixed()
    fe, fp, oh = c.wall_ledger()
    assert list(gh) == list(oh)
    assert [round(x * 2**24) for x in ge] == list(oe)
    assert [round(x * 2**24) for x in gp] == list(op)
    for w in range(7):  # the f64 sums in particle order, within 2^-25 per event
        events = max(int(oh[w]), 1)
        assert abs(ge[w] - fe[w]) <= events * 2.0**-25 + 1e-12
    return sum(gh)


def _same_compartment_ledger(g, c):
    """GpuEngine::read_compartment_ledger against the oracle's walls::CompartmentLedger (integer
    sums per slot and compartment along the wall)."""
    ge, gp, gh = g.read_compartment_ledger()
    oe, op, oh = c.compartment_ledger_fixed()
    assert ge.shape == oe.shape
    assert np.array_equal(gh, oh)
    assert np.array_equal(np.round(ge * 2**24).astype(np.int64), oe)
    assert np.array_equal(np.round(gp * 2**24).astype(np.int64), op)
    return oh


def _gas_in_walls(O, n, density, seed, kind, gravity):
    """boundaries.rs:6-35: a WCA gas in a box walled on both axes (hard or soft), with gravity."""
    w = Wall.hard() if kind == "hard" else Wall.soft()
    sys_ = System(box_for(n, density, 1.0), 0.005, Pair.wca(), [1.0]).with_walls(1, w, w).with_walls(0, w, w)
    sys_.with_gravity([0.0, -gravity])
    return sys_, O.fluid(sys_, n, 1.0, seed)


@pytest.mark.parametrize("kind", ["hard", "soft"])
@pytest.mark.parametrize("mode", ["cells", "verlet"])
def test_walls_with_gravity_follow_the_oracle_and_reverse(O, kind, mode):
    """boundaries.rs:12-35 on the GPU: 400 WCA discs between hard (soft) walls on both axes under
    gravity, 2000 steps equal IntEngine's bit for bit with the same ledger; then reversed, 2000
    steps and reversed again, the initial state exactly."""
    n = 400
    sys_, s0 = _gas_in_walls(O, n, 0.3, 1, kind, 0.5)
    m = ForceMode.cell_list() if mode == "cells" else ForceMode.verlet_with_skin(sys_, n, 0.3)
    c = O.IntEngine(sys_, s0)
    with GpuEngine(sys_, s0, m) as g:
        g.step(2000)
        c.step(2000)
        assert g.read_state() == c.state
        hits = _same_ledger(g, c)
        if kind == "hard":
            assert hits > 100
        else:
            assert sum(g.read_ledger()[1]) > 1.0  # the soft walls were pushed
        kg, _ = g.kicks()
        kc, _ = c.kicks()
        assert np.array_equal(kg, kc)
        g.reverse()
        g.step(2000)
        g.reverse()
        assert g.read_state() == s0


@pytest.mark.parametrize("mode", ["cells", "verlet"])
def test_wca_mixture_with_walls_and_gravity_follows_the_oracle(O, mode):
    """md-ref/tests/fast_path.rs:27-46 on the GPU: a WCA mixture of three masses (1, 4, 30) and two
    sizes (the heavy species 2 sigma from the others, 3 among themselves), hard walls on x, soft
    on y, gravity 0.01; the small particles within 2 sigma of a big one removed. 300 steps equal
    IntEngine<f32>'s bit for bit with the same ledger."""

    def wca(s):
        return Pair(1.0, s, s * 2 ** (1 / 6))

    sys_ = System(box_for(1500, 0.3, 1.5), 0.005, wca(1.0), [1.0, 4.0, 30.0])
    sys_.with_pair(0, 2, wca(2.0)).with_pair(1, 2, wca(2.0)).with_pair(2, 2, wca(3.0))
    sys_.with_walls(0, Wall.hard(), Wall.hard()).with_walls(1, Wall.soft(), Wall.soft()).with_gravity([0.0, -0.01])
    st = O.fluid(sys_, 1500, 1.0, 2)
    st.species[:] = [2 if i % 50 == 0 else i % 2 for i in range(1500)]
    big = st.pos[st.species == 2]
    d2 = (((big[None, :, :] - st.pos[:, None, :]).astype(np.float64) / ONE) ** 2).sum(-1)
    keep = (st.species == 2) | (d2 > 4.0).all(1)
    s0 = State(st.pos[keep].copy(), st.vel[keep].copy(), st.species[keep].copy())
    n = s0.n()
    m = ForceMode.cell_list() if mode == "cells" else ForceMode.verlet_with_skin(sys_, n, 0.3)
    c = O.IntEngine(sys_, s0)
    with GpuEngine(sys_, s0, m) as g:
        g.step(300)
        c.step(300)
        assert g.read_state() == c.state
        _same_ledger(g, c)


def test_soft_walls_energy_matches_the_oracle(O):
    """The instruments with soft walls (the walls' WCA potential in forces(), int_engine.rs:
    203-227): the GPU's kicks equal the oracle's; the potential within 1e-5 relative (the oracle
    sums each particle's f32 pair energies in f32, as IntEngine<f32> does; the GPU sums them more
    exactly), the kinetic energy within 1e-9."""
    n = 600
    w = Wall.soft()
    sys_ = System(box_for(n, 0.5, 1.5), 0.005, Pair.lj(2.5), [1.0]).with_walls(0, w, w)
    s0 = O.fluid(sys_, n, 1.0, 3)
    c = O.IntEngine(sys_, s0)
    c.step(300)
    st = c.state
    with GpuEngine(sys_, st, ForceMode.verlet_with_skin(sys_, n, 0.3)) as g:
        kg, _ = g.kicks()
        ke, pe = g.energy()
    kc, _ = c.kicks()
    assert np.array_equal(kg, kc)
    oke, ope = c.energy()
    assert abs(pe - ope) <= 1e-5 * abs(ope)
    assert abs(ke - oke) <= 1e-9 * abs(oke)


@pytest.mark.parametrize("dim", [2, 3])
def test_thermal_walls_follow_the_oracle(O, dim):
    """Non-interacting particles (a 0.1-sigma pair) at up to 0.25 sigma per step between a hot and
    a cold thermal wall (and, in 3D, hard walls on z): every collision draws on (id, step clock)
    as walls::thermal_velocity / three::thermal_velocity do; 600 steps equal the oracle's bit for
    bit, with the same ledger."""
    L, n = 12.0, 64
    tiny = Pair(1.0, 0.1, 0.1 * 2 ** (1 / 6))
    box = [int(L * ONE)] * dim
    hot, cold = Wall.thermal(2.0), Wall.thermal(0.5)
    if dim == 2:
        sys_ = System(box, 0.005, tiny, [1.0, 3.0]).with_walls(0, hot, cold)
    else:
        sys_ = System3(box, 0.005, tiny, [1.0, 3.0]).with_walls(0, hot, cold).with_walls(2, Wall.hard(), Wall.hard())
    sys_.seed = 0x2468_ACE0_1357
    rng = np.random.default_rng(5)
    pos = ((rng.random((n, dim)) * (L - 2) + 1) * ONE).astype(np.int64)
    vel = (rng.choice([-1, 1], (n, dim)) * rng.uniform(0.05, 0.25, (n, dim)) * ONE).astype(np.int32)
    sp = np.array([k % 2 for k in range(n)], np.uint32)
    st = (State if dim == 2 else State3)(pos, vel, sp)
    cls = GpuEngine if dim == 2 else GpuEngine3
    c = O.IntEngine(sys_, st)
    with cls(sys_, st, ForceMode.cell_list()) as g:
        for _ in range(6):
            g.step(100)
            c.step(100)
            assert g.read_state() == c.state
        hits = _same_ledger(g, c)
    assert hits > 50


def test_thermal_walls_set_the_temperature(O):
    """boundaries.rs:91-110 on the GPU: a dilute WCA gas at T = 0.5 between thermal walls at 1.5
    reaches T = 1.5 within 0.06, taking more than 0.5 epsilon per particle from the walls."""
    n = 150
    w = Wall.thermal(1.5)
    sys_ = System(box_for(n, 0.1, 1.0), 0.005, Pair.wca(), [1.0]).with_walls(0, w, w).with_walls(1, w, w)
    s0 = O.fluid(sys_, n, 0.5, 4)
    with GpuEngine(sys_, s0, ForceMode.cell_list()) as g:
        g.step(40000)
        t = 0.0
        for _ in range(200):
            g.step(100)
            ke, _ = g.energy()
            t += ke / n / 200  # 2D: T = KE / N (kT per particle of 2 degrees of freedom)
        heat = sum(g.read_ledger()[0])
    assert abs(t - 1.5) < 0.06, t
    assert heat > 0.5 * n


def test_walled_liquid_3d_follows_the_oracle(O):
    """A 3D LJ liquid (N = 20,000, rho 0.8) between soft walls on z, Verlet lists: 300 steps equal
    IntEngine3's bit for bit, with the same ledger, and a frame's RDF equals the oracle's counts
    (plain differences across the walled axis)."""
    n = 20_000
    sys3 = System3(cube_for(n, 0.8), 0.005, Pair.lj(2.5), [1.0]).with_walls(2, Wall.soft(), Wall.soft())
    s0 = O.fcc_maxwell(sys3, n, 1.0, 7, jitter=0.05)
    # keep the lattice a sigma clear of the walls: squeeze z into [1, L - 1)
    L = sys3.box_len[2]
    s0.pos[:, 2] = (ONE + s0.pos[:, 2].astype(np.float64) / L * (L - 2 * ONE)).astype(np.int64)
    c = O.IntEngine(sys3, s0, threads=8)
    with GpuEngine3(sys3, s0, ForceMode.verlet_with_skin(sys3, n, 0.3)) as g:
        g.step(300)
        c.step(300)
        assert g.read_state() == c.state
        _same_ledger(g, c)
        f, rdf, _ = g.observe(rdf_bins=100, rdf_rmax=3.0)
    assert np.array_equal(rdf, O.rdf(sys3, c.state, 100, 3.0))


# ---------------------------------------------------------------- membranes and compartments (2D)
@pytest.mark.parametrize("diathermal", [False, True])
@pytest.mark.parametrize("mode", ["cells", "verlet"])
def test_compartments_follow_the_oracle_and_reverse(O, diathermal, mode):
    """md-ref/tests/boundaries.rs:154-181 on the GPU: 16 x 16 compartments of 8 sigma between hard
    walls, 6 particles each; insulating (pairs in different boxes do not interact) or diathermal.
    1500 steps equal IntEngine's bit for bit; every particle is still in its own box; the run
    reverses exactly."""
    from test_oracle import _compartment_fluid

    side = 8 * ONE
    sys_ = System([16 * side, 16 * side], 0.005, Pair.wca(), [1.0])
    sys_.with_walls(0, Wall.hard(), Wall.hard()).with_walls(1, Wall.hard(), Wall.hard())
    sys_.with_compartments(0, 3).with_compartments(1, 3)
    if diathermal:
        sys_.with_diathermal_compartments()
    s0 = _compartment_fluid(O, sys_, 6, 1.0, 7)
    home = [sys_.compartment_of(p) for p in s0.pos]
    n = s0.n()
    m = ForceMode.cell_list() if mode == "cells" else ForceMode.verlet_with_skin(sys_, n, 0.3)
    c = O.IntEngine(sys_, s0)
    with GpuEngine(sys_, s0, m) as g:
        g.step(1500)
        c.step(1500)
        got = g.read_state()
        assert got == c.state
        assert [sys_.compartment_of(p) for p in got.pos] == home
        _same_ledger(g, c)
        hits = _same_compartment_ledger(g, c)
        assert hits.shape == (7, 16) and (hits[:4].sum(axis=1) > 0).all()  # every outer wall, per box along it
        g.reverse()
        g.step(1500)
        g.reverse()
        assert g.read_state() == s0


@pytest.mark.parametrize("mode,pores", [("cells", False), ("verlet", False), ("verlet", True)])
def test_membrane_follows_the_oracle(O, mode, pores):
    """md-ref/tests/boundaries.rs:241-268 on the GPU: soft walls on x, a membrane at the middle
    blocking species 1 (the solute, 20% of the right half), optionally with pores 0.5 sigma wide
    every 2 sigma: 3000 steps equal IntEngine's bit for bit with the same ledger (membrane faces 4
    and 5); without pores no solute crossed."""
    from micrographia_gb300.workloads import uniform

    from micrographia_gb300 import to_f64

    n = 1200
    sys_ = System(box_for(n, 0.4, 2.0), 0.005, Pair.wca(), [1.0, 1.0]).with_walls(0, Wall.soft(), Wall.soft())
    half = sys_.box_f64()[0] / 2.0
    sys_.with_membrane(0, half, [1])
    if pores:
        sys_.with_pores(1, 0.5)
    s0 = O.fluid(sys_, n, 1.0, 13)
    for i in range(n):
        if to_f64(int(s0.pos[i, 0])) > half + 1.0 and uniform(13, 3, i) < 0.2:
            s0.species[i] = 1
    m = ForceMode.cell_list() if mode == "cells" else ForceMode.verlet_with_skin(sys_, n, 0.3)
    c = O.IntEngine(sys_, s0)
    with GpuEngine(sys_, s0, m) as g:
        g.step(3000)
        c.step(3000)
        st = g.read_state()
        assert st == c.state
        _same_ledger(g, c)
        _same_compartment_ledger(g, c)
        hits_right = g.read_ledger()[2][5]
    if not pores:
        assert hits_right > 20  # the solute hit the membrane from the right
        assert all(to_f64(int(p)) > half - 0.5 for p in st.pos[st.species == 1, 0])


# ---------------------------------------------------------------- pistons (2D)
def _piston_gas(O, n, density, drive, seed):
    """md-ref/tests/boundaries.rs:270-285: a WCA gas under a piston (soft floor, hard roof at twice
    box_for's height, the piston starting at half of it and stopping at 2 sigma)."""
    from test_oracle import _gas_under_piston

    return _gas_under_piston(O, n, density, drive, seed)


@pytest.mark.parametrize("mode", ["cells", "verlet"])
def test_driven_piston_follows_the_oracle_and_reverses(O, mode):
    """boundaries.rs:287-298 on the GPU: 500 particles under a piston driven down at 0.5 sigma/tau:
    2000 steps equal IntEngine<f32>'s bit for bit (state, piston height, velocity and work, and
    the ledger); reversed, 2000 steps and reversed again, the initial state and height exactly."""
    from micrographia_gb300 import Piston

    sys_, s0 = _piston_gas(O, 500, 0.3, Piston.speed_drive(-0.5), 16)
    n = s0.n()
    m = ForceMode.cell_list() if mode == "cells" else ForceMode.verlet_with_skin(sys_, n, 0.3)
    c = O.IntEngine(sys_, s0)
    with GpuEngine(sys_, s0, m) as g:
        w0 = g.piston()[0]
        assert w0 == c.piston()[0]
        g.step(2000)
        c.step(2000)
        assert g.read_state() == c.state
        assert g.piston() == c.piston()[:3]
        assert g.piston()[0] < w0
        _same_ledger(g, c)
        kg, peg = g.kicks()
        kc, pec = c.kicks()
        assert np.array_equal(kg, kc)
        g.reverse()
        g.step(2000)
        g.reverse()
        assert g.read_state() == s0
        assert g.piston()[0] == w0


def test_free_piston_follows_the_oracle_and_balances_the_pressure(O):
    """boundaries.rs:300-319 on the GPU: a free piston (mass 50, 15 eps/sigma down) over 600
    particles; 3000 steps equal IntEngine<f32>'s bit for bit (the piston's kicks come from the
    gas's force summed in 2^-16 units, so in any order the same); then, after 10,000 steps, the
    floor's time-averaged pressure over 60,000 steps equals the external pressure within 5%."""
    from micrographia_gb300 import Piston

    force = 15.0
    sys_, s0 = _piston_gas(O, 600, 0.2, Piston.free(50.0, force), 17)
    width = sys_.box_f64()[0]
    c = O.IntEngine(sys_, s0)
    with GpuEngine(sys_, s0, ForceMode.verlet_with_skin(sys_, s0.n(), 0.3)) as g:
        g.step(3000)
        c.step(3000)
        assert g.read_state() == c.state
        assert g.piston() == c.piston()[:3]
        g.step(7000)
        before = g.read_ledger()[1][2]
        steps = 60000
        g.step(steps)
        p_bottom = (g.read_ledger()[1][2] - before) / (steps * sys_.dt * width)
    assert abs(p_bottom / (force / width) - 1.0) < 0.05, p_bottom


def test_driven_piston_with_a_bath_follows_the_oracle(O):
    """A piston driven up at 0.3 sigma/tau over a gas in an Andersen bath (T 1.2, rate 2 per tau):
    redrawn particles take the piston's affine flow (int_engine.rs:282-286); 1500 steps equal
    IntEngine<f32>'s bit for bit, with the same ledger (the bath's energy included)."""
    from micrographia_gb300 import Piston

    sys_, s0 = _piston_gas(O, 400, 0.3, Piston.speed_drive(0.3), 19)
    sys_.with_thermostat(1.2, 2.0)
    c = O.IntEngine(sys_, s0)
    with GpuEngine(sys_, s0, ForceMode.cell_list()) as g:
        for _ in range(3):
            g.step(500)
            c.step(500)
            assert g.read_state() == c.state
            assert g.piston() == c.piston()[:3]
        _same_ledger(g, c)


def test_piston_page_commands(O):
    """GpuEngine::read_piston and set_piston_speed (engine.rs:936-961): the gas's force on the
    piston in the last step equals the oracle's; a new speed set on both between steps keeps the
    runs bit-identical."""
    from micrographia_gb300 import Piston
    from test_oracle import _gas_under_piston

    sys_, s0 = _gas_under_piston(O, 500, 0.3, Piston.speed_drive(-0.5), 16)
    c = O.IntEngine(sys_, s0)
    with GpuEngine(sys_, s0, ForceMode.verlet_with_skin(sys_, s0.n(), 0.3)) as g:
        g.step(600)
        c.step(600)
        h, v, f, work = g.read_piston()
        w, vi, cwork, cf = c.piston()
        assert (h, v) == (w / 2**32, vi / 2**32 / sys_.dt) and work == cwork
        assert f == cf and f > 0.0
        g.set_piston_speed(0.25)
        c.set_piston_speed(0.25)
        g.step(600)
        c.step(600)
        assert g.read_state() == c.state
        assert g.piston() == c.piston()[:3]


def _liquid3(n, density, t, walls):
    """crates/md/tests/three.rs:15-31: an FCC liquid (jitter 0.05, seed 7) with Maxwell velocities
    (seed 3); with hard walls on z, the sites kept half a sigma clear of them."""
    from micrographia_gb300 import DT, ONE, State3, System3, init

    sys3 = System3(cube_for(n, density), DT, Pair.lj(2.5), [1.0])
    if walls:
        sys3.with_walls(2, Wall.hard(), Wall.hard())
    pos = init.fcc_maxwell(sys3, n, t, 7, jitter=0.05).pos
    if walls:
        pos[:, 2] = np.clip(pos[:, 2], ONE // 2, sys3.box_len[2] - ONE // 2)
    sp = np.zeros(n, np.uint32)
    return sys3, State3(pos, init.maxwell(sys3, sp, t, 3), sp)


def test_bath_and_hot_walls_set_the_temperature_3d():
    """three.rs:113-133: a 3D Andersen bath at 1.6 brings a liquid (4000 at density 0.5, T 0.8) to
    kT 1.6 within 0.06 in 4000 steps; heat-bath walls at 2.0 on z bring a thin gas (2000 at 0.05)
    to kT 2.0 within 0.1 in 60000 steps, the walls' ledger showing the energy they gave."""
    sys3, s = _liquid3(4000, 0.5, 0.8, False)
    sys3.with_thermostat(1.6, 2.0)
    with GpuEngine3(sys3, s) as g:
        g.step(4000)
        t = g.read_kinetic_total() / (1.5 * 4000)
    assert abs(t - 1.6) < 0.06, t
    sys3, s = _liquid3(2000, 0.05, 0.5, True)
    sys3.with_walls(2, Wall.thermal(2.0), Wall.thermal(2.0))
    with GpuEngine3(sys3, s) as g:
        g.step(60000)
        t = g.read_kinetic_total() / (1.5 * 2000)
        e, _, h = g.read_ledger()
    assert abs(t - 2.0) < 0.1, t
    assert h[4] + h[5] > 0 and e[4] + e[5] > 0
