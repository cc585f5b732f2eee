"""The oracle against the reference's own known answers and property tests (CPU only).

Pins: Random123 Threefry KATs (crates/gpu-prims/src/threefry.rs:52-70), GOLDEN_INT_HASH
(crates/md/src/checks.rs:155-167, crates/md/tests/integer.rs:250-264), fixed-point separation
identities (crates/md-core/src/fixed.rs:74-99, crates/md-ref/tests/fast_path.rs:56-79), and the
md-ref property tests (crates/md-ref/tests/physics.rs, fast_path.rs)."""

import json
import math
import os

import numpy as np
import pytest

from micrographia_gb300 import ONE, Pair, State, System, System3, box_for, cube_for, fcc_cells, to_f64

HERE = os.path.dirname(os.path.abspath(__file__))
VEC = json.load(open(os.path.join(HERE, "golden", "reference_vectors.json")))


def wca_fluid(O, n, density, t, seed, masses=(1.0,)):
    sys_ = System(box_for(n, density, 1.0), 0.005, Pair.wca(), list(masses))
    return sys_, O.fluid(sys_, n, t, seed)


def test_threefry_known_answers(O):
    assert len(VEC["threefry_kat"]) == 9
    for k in VEC["threefry_kat"]:
        assert O.threefry(k["ctr"], k["key"], k["rounds"]) == k["want"], k


def test_golden_int_hash(O):
    """All-integer forces, 3000-particle binary LJ mixture, 1000 steps: the reference's hash."""
    sys_ = System(box_for(3000, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0, 2.0]).with_pair(0, 1, Pair(0.7, 1.05, 2.5))
    s = O.fluid(sys_, 3000, 1.0, 2026)
    s.species[::4] = 1
    s.vel = O.maxwell(sys_, s.species, 1.0, 2026)
    e = O.IntEngine(sys_, s, f64=True, integer=True)
    e.step(1000)
    assert e.hash() == int(VEC["golden_int_hash"], 16)


def test_separation_identities(O):
    # fixed.rs:90-98
    for d in [1, 15, 16, 17, ONE, ONE + 7, 3 * ONE // 2, 8 * ONE - 1, 123_456_789]:
        a, b = O.sep_f32(-d), O.sep_f32(d)
        assert np.float32(a).tobytes() == np.float32(-b).tobytes()
    assert O.sep_f32(8 * ONE) is None
    assert O.sep_f32(-8 * ONE) is not None
    assert abs(O.sep_f32(ONE + ONE // 4) - 1.25) < 1e-7


def test_sep_near_matches_sep_f32(O):
    # fast_path.rs:56-79 (xorshift over four ranges, 2M draws)
    lim = 8 * ONE
    x = 0x9E3779B97F4A7C15
    m64 = (1 << 64) - 1
    checked = 0
    for k in range(200_000):
        x ^= (x << 13) & m64
        x ^= x >> 7
        x ^= (x << 17) & m64
        r = k % 4
        if r == 0:
            d = (x % (2 * lim)) - lim
        elif r == 1:
            d = (x % 1024) - 512
        elif r == 2:
            d = ((x % 64) - 32) << 32
        else:
            d = (x % (2 * lim)) - lim + 1
        if d >= lim or d < -lim:
            continue
        a = np.float32(O.lib().oracle_sep_near(d)).tobytes()
        b = np.float32(O.sep_f32(d)).tobytes()
        assert a == b, d
        checked += 1
    assert checked > 150_000


def test_box_helpers_match_host_mirror(O):
    for n, rho, asp in [(4096, 0.7, 1.0), (3000, 0.6, 1.0), (16_777_216, 0.2125, 4.0), (500, 0.7, 2.0)]:
        assert O.box_for(n, rho, asp) == box_for(n, rho, asp)
    for n, rho in [(1_048_576, 0.8442), (4000, 0.8), (500, 1.0)]:
        b = cube_for(n, rho)
        assert O.cube_for(n, rho) == b
        assert O.fcc_cells(n, b) == fcc_cells(n, b)
    assert fcc_cells(4 * 64**3, cube_for(4 * 64**3, 0.8442)) == [64, 64, 64]
    assert O.lib().oracle_wca_rc() == Pair.wca().rc
    for p in [Pair.lj(2.5), Pair.wca(), Pair(0.7, 1.05, 2.5)]:
        assert O.lib().oracle_pair_shift(p.eps, p.sigma, p.rc) == p.shift()


def test_zero_sum_is_exact_and_temperature(O):
    # init.rs:175-182
    sys_, s = wca_fluid(O, 1000, 0.5, 1.3, 9)
    assert s.velocity_sum() == [0, 0]
    t = O.half_step_kinetic(sys_, s) / (s.n() - 1)
    assert abs(t - 1.3) < 0.1


def test_lattice_inside_box(O):
    # init.rs:185-189
    b = box_for(500, 0.7, 2.0)
    sys_ = System(b, 0.005, Pair.wca(), [1.0])
    s = O.fluid(sys_, 500, 1.0, 1)
    assert (s.pos >= 0).all() and (s.pos[:, 0] < b[0]).all() and (s.pos[:, 1] < b[1]).all()


def test_fcc_geometry_and_3d_maxwell(O):
    # three.rs:410-446
    n = 4 * 5 * 5 * 5
    b = cube_for(n, 1.0)
    assert fcc_cells(n, b) == [5, 5, 5]
    sys3 = System3(b, 0.005, Pair.wca(), [1.0])
    s = O.fcc_maxwell(sys3, n, 1.0, 1, jitter=0.0)
    p = s.pos.astype(np.float64) / ONE
    l = to_f64(b[0])
    d = p[:50, None, :] - p[None, :, :]
    d -= l * np.round(d / l)
    r = np.sqrt((d**2).sum(-1))
    r[r == 0] = 1e9
    assert abs(r.min() - 4 ** (1 / 3) / math.sqrt(2)) < 1e-6
    n = 4000
    sys3 = System3(cube_for(n, 0.5), 0.005, Pair.wca(), [1.0])
    s = O.fcc_maxwell(sys3, n, 1.3, 2, jitter=0.0)
    assert s.velocity_sum() == [0, 0, 0]
    v = s.vel.astype(np.float64) / ONE / 0.005
    assert abs(0.5 * (v**2).sum() / (1.5 * n) - 1.3) < 0.05
    vel = O.set_temperature(sys3, s, 0.7)
    v = vel.astype(np.float64) / ONE / 0.005
    assert abs(0.5 * (v**2).sum() / (1.5 * (n - 1)) - 0.7) < 1e-3
    assert vel.astype(np.int64).sum(axis=0).tolist() == [0, 0, 0]


def test_reversal_is_exact(O):
    # physics.rs:17-37
    for f64 in (False, True):
        sys_, s0 = wca_fluid(O, 400, 0.6, 1.0, 1)
        e = O.IntEngine(sys_, s0, f64=f64)
        e.step(1500)
        assert e.state != s0
        e.reverse()
        e.step(1500)
        e.reverse()
        assert e.state == s0
        assert e.steps == 0


def test_one_bit_flip_breaks_reversal(O):
    # physics.rs:39-51
    sys_, s0 = wca_fluid(O, 400, 0.6, 1.0, 2)
    e = O.IntEngine(sys_, s0)
    e.step(3000)
    st = e.state
    st.flip_bit(0, 0, 0)
    e.set_state(st)
    e.reverse()
    e.step(3000)
    e.reverse()
    differ, mx = e.state.position_difference(s0, sys_)
    assert differ > 300 and mx > 0.5


def test_storage_order_does_not_matter(O):
    # physics.rs:53-69
    sys_, s0 = wca_fluid(O, 500, 0.6, 1.0, 3)
    perm = np.random.default_rng(11).permutation(500)
    a = O.IntEngine(sys_, s0)
    b = O.IntEngine(sys_, s0.permuted(perm))
    a.step(500)
    b.step(500)
    assert b.state.unpermuted(perm) == a.state


def test_momentum_is_exactly_conserved(O):
    sys_, s0 = wca_fluid(O, 500, 0.6, 1.0, 4)
    assert s0.velocity_sum() == [0, 0]
    e = O.IntEngine(sys_, s0)
    for _ in range(5):
        e.step(100)
        assert e.state.velocity_sum() == [0, 0]


def test_integer_and_float_engines_agree_initially(O):
    # physics.rs:109-127
    sys_, s0 = wca_fluid(O, 400, 0.6, 1.0, 6)
    i = O.IntEngine(sys_, s0, f64=True)
    f = O.FloatEngine(sys_, s0)
    i.step(20)
    f.step(20)
    p = i.state.pos.astype(np.float64) / ONE
    q = f.positions()
    b = np.array(sys_.box_f64())
    d = np.abs(p - q)
    d = np.minimum(d, b - d)
    assert d.max() < 1e-7


def test_f32_kicks_match_f64_kicks(O):
    # physics.rs:129-146
    sys_, s0 = wca_fluid(O, 1000, 0.7, 1.0, 7)
    k32, pe32 = O.IntEngine(sys_, s0).kicks()
    k64, pe64 = O.IntEngine(sys_, s0, f64=True).kicks()
    rel = math.sqrt(((k32.astype(np.float64) - k64) ** 2).sum() / (k64.astype(np.float64) ** 2).sum())
    assert rel < 1e-5
    assert abs((pe32 - pe64) / pe64) < 1e-5


def test_fast_path_matches_the_reference(O):
    # fast_path.rs:20-54 (the periodic cases)
    sys_ = System(box_for(2000, 0.7, 1.0), 0.005, Pair.lj(2.5), [1.0])
    st = O.fluid(sys_, 2000, 0.8, 1)
    a, b = O.IntEngine(sys_, st, fast=True), O.IntEngine(sys_, st, fast=False)
    a.step(300)
    b.step(300)
    assert a.state == b.state
    ea, eb = a.kicks()[1], b.kicks()[1]
    assert abs(ea - eb) < 1e-4 * max(abs(eb), 1.0)
    # a periodic WCA mixture of three masses and two sizes
    wca = lambda s: Pair(1.0, s, s * 2 ** (1 / 6))
    sys_ = System(box_for(1500, 0.3, 1.5), 0.005, wca(1.0), [1.0, 4.0, 30.0]).with_pair(0, 2, wca(2.0)).with_pair(1, 2, wca(2.0)).with_pair(2, 2, wca(3.0))
    st = O.fluid(sys_, 1500, 1.0, 2)
    for i in range(1500):
        st.species[i] = 2 if i % 50 == 0 else i % 2
    big = st.pos[st.species == 2].astype(np.float64) / ONE
    keep = [i for i in range(1500) if st.species[i] == 2 or (((big - st.pos[i] / ONE) ** 2).sum(axis=1) > 4.0).all()]
    st = type(st)(st.pos[keep], st.vel[keep], st.species[keep])
    a, b = O.IntEngine(sys_, st, fast=True), O.IntEngine(sys_, st, fast=False)
    a.step(300)
    b.step(300)
    assert a.state == b.state


def test_integer_kicks_are_antisymmetric_and_accurate(O):
    # table.rs:113-136
    import ctypes as C

    sys_ = System(box_for(100, 0.5, 1.0), 0.005, Pair.lj(2.5), [1.0])
    c = sys_.to_c()
    worst = 0.0
    for k in range(0, 2000, 7):
        r = 0.8 + 1.69 * k / 2000.0
        a = 0.3 + k * 0.001
        d = (C.c_int64 * 2)(int(round(r * math.cos(a) * ONE)), int(round(r * math.sin(a) * ONE)))
        dm = (C.c_int64 * 2)(-d[0], -d[1])
        ki, kj = (C.c_int32 * 2)(), (C.c_int32 * 2)()
        assert O.lib().oracle_int_kick(C.byref(c), 0, 0, d, ki) == 1
        assert O.lib().oracle_int_kick(C.byref(c), 0, 0, dm, kj) == 1
        assert [ki[0], ki[1]] == [-kj[0], -kj[1]]
        f = sys_.pair(0, 0).f_over_r(r * r) * sys_.kick_coeff(0)
        exact = [-f * r * math.cos(a), -f * r * math.sin(a)]
        for ax in range(2):
            worst = max(worst, abs(ki[ax] - exact[ax]) / (20.0 + 1e-5 * abs(exact[ax])))
    assert worst < 1.0


def test_cells_and_lists_are_consistent(O):
    """The Verlet-list restatement holds every pair within rc (the list invariant)."""
    sys_ = System(box_for(1500, 0.7, 1.0), 0.005, Pair.lj(2.5), [1.0])
    st = O.fluid(sys_, 1500, 1.0, 3)
    lists = O.verlet_lists(sys_, st, 0.3)
    p = st.pos.astype(np.float64) / ONE
    b = np.array(sys_.box_f64())
    for i in range(0, 1500, 37):
        d = p - p[i]
        d -= b * np.round(d / b)
        r = np.sqrt((d**2).sum(1))
        within = set(np.nonzero((r < 2.5) & (np.arange(1500) != i))[0].tolist())
        assert within <= set(lists[i].tolist())
        assert all(r[j] < 2.81 for j in lists[i])


def test_cell_list_is_a_stable_counting_sort(O):
    sys_ = System(box_for(3000, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0])
    st = O.fluid(sys_, 3000, 1.0, 5)
    dims = sys_.cells_for(2.5)
    keys, start, items = O.cell_list(sys_, st, dims)
    want = np.argsort(keys, kind="stable")
    assert (items == want).all()
    assert start[-1] == 3000 and (np.diff(start.astype(np.int64)) >= 0).all()


def test_rescale_thermostat_is_exact(O):
    sys_, s = wca_fluid(O, 2000, 0.5, 1.7, 4)
    vel = O.set_temperature(sys_, s, 0.45, exact=True)
    assert vel.astype(np.int64).sum(axis=0).tolist() == [0, 0]
    s2 = type(s)(s.pos, vel, s.species)
    t = O.exact_kinetic(sys_, s2) / (s.n() - 1)
    assert abs(t - 0.45) < 1e-3


def _rdf_brute(sys_, st, bins, rmax):
    """Every unordered pair's exact minimum-image separation, binned as floor(r * bins / rmax)."""
    d = sys_.DIM
    pos = st.pos.reshape(-1, d).astype(np.int64)
    box = np.array(sys_.box_len, np.int64)
    half = box // 2
    r2 = np.zeros((len(pos), len(pos)))
    for a in range(d):
        dd = pos[None, :, a] - pos[:, None, a]
        dd = np.where(dd >= half[a], dd - box[a], np.where(dd < -half[a], dd + box[a], dd))
        f = dd.astype(np.float64) * (1.0 / ONE)
        r2 = r2 + f * f
    r = np.sqrt(r2) * (bins / rmax)
    iu = np.triu_indices(len(pos), 1)
    r = r[iu]
    r = r[r < bins]
    return np.bincount(r.astype(np.int64), minlength=bins).astype(np.uint64)


@pytest.mark.parametrize("rmax", [4.0, 7.0])
def test_rdf_counts_every_pair_once(O, rmax):
    """Cell-list RDF (range under a third of the box) and the all-pairs form for a wider range
    both equal a brute-force count."""
    sys_ = System(box_for(200, 0.5, 1.0), 0.005, Pair.lj(2.5), [1.0])
    st = O.fluid(sys_, 200, 1.0, 9)
    assert (sys_.box_f64()[0] / rmax >= 3) == (rmax == 4.0)
    assert np.array_equal(O.rdf(sys_, st, 90, rmax), _rdf_brute(sys_, st, 90, rmax))


def test_to_step_displacement_rounds_like_rust(O):
    """System::to_step_displacement: f64 round half away from zero, saturating, NaN -> 0."""
    s = System(box_for(100, 0.7, 1.0), 2.0**-32, Pair.lj(2.5), [1.0])  # v dt 2^32 = v
    assert [O.to_step_displacement(s, v) for v in (0.5, -0.5, 1.5, -2.5, 0.49999999999999994)] == [1, -1, 2, -3, 0]
    assert O.to_step_displacement(s, 3e9) == 2**31 - 1 and O.to_step_displacement(s, -3e9) == -(2**31)
    assert O.to_step_displacement(s, float("nan")) == 0


def _andersen_py(sys_, i, clock, s, p, dim):
    """walls::andersen (walls.rs:113-133) / three::andersen (three.rs:247-265) restated in Python
    (math.log/cos/sin are the platform libm, as Rust's f64 methods are): the new velocity in
    sigma/tau, or None."""
    from micrographia_gb300.workloads import threefry2x32

    th = sys_.thermostat
    if not (th.species >> s) & 1 or (dim == 2 and not th.region[0] <= p[th.axis] < th.region[1]):
        return None
    if dim == 3 and (sys_.pinned >> s) & 1:
        return None
    k0, k1 = sys_.seed & 0xFFFFFFFF, ((sys_.seed >> 32) ^ 0x5448524D) & 0xFFFFFFFF
    unit = lambda w: ((w << 21) & ((1 << 53) - 1)) * (1.0 / (1 << 53))
    r = threefry2x32(i, clock, k0, k1)
    if unit(r[0]) >= th.rate * sys_.dt:
        return None
    r2 = threefry2x32(i, clock, k0, k1 ^ 1)
    sd = math.sqrt(th.t / sys_.masses[s])
    rad = math.sqrt(-2.0 * math.log(1.0 - unit(r[1])))
    a = 2.0 * math.pi * unit(r2[0])
    out = [sd * rad * math.cos(a), sd * rad * math.sin(a)]
    if dim == 3:
        r3 = threefry2x32(i, clock, k0, k1 ^ 2)
        out.append(sd * math.sqrt(-2.0 * math.log(1.0 - unit(r3[0]))) * math.cos(2.0 * math.pi * unit(r3[1])))
    return out


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_bath_draws_match_a_python_restatement(O, dim):
    """Particles too far apart to interact: after each step a particle's velocity is its bath
    draw for (id, clock) (plus the fan's drift in 2D) or unchanged; the oracle's C++ bath equals
    an independent Python restatement of the reference's, draw for draw."""
    from micrographia_gb300 import State, State3, System3 as S3

    n, L = 6, 60.0
    box = [int(L * ONE)] * dim
    if dim == 2:
        sys_ = System(box, 0.005, Pair.lj(2.5), [1.0, 2.5]).with_thermostat(0.9, 120.0).with_fan(0b11, 0.0, 45.0, 0.25)
    else:
        sys_ = S3(box, 0.005, Pair.lj(2.5), [1.0, 2.5]).with_thermostat(0.9, 120.0)
    sys_.seed = 0x1234_5678_9ABC
    pos = np.array([[(10 * k + 3) * ONE] * dim for k in range(n)], np.int64)
    sp = np.array([k % 2 for k in range(n)], np.uint32)
    st = (State if dim == 2 else State3)(pos, np.zeros((n, dim), np.int32), sp)
    c = O.IntEngine(sys_, st)
    drift = sys_.to_step_displacement(0.25) if dim == 2 else 0
    hits = 0
    for clock in range(40):
        before = c.state
        c.step(1)
        after = c.state
        for i in range(n):
            u = _andersen_py(sys_, i, clock, int(sp[i]), before.pos[i], dim)
            if u is None:
                assert list(after.vel[i]) == list(before.vel[i])
            else:
                want = [sys_.to_step_displacement(x) for x in u]
                if dim == 2:
                    want[0] = (want[0] + drift + 2**31) % 2**32 - 2**31
                assert list(after.vel[i]) == want, (clock, i)
                hits += 1
    assert hits > 40 * n // 4  # rate dt = 0.6; in 2D the fan's x range holds 5 of the 6
    assert c.ledger()[2] == hits and c.ledger()[3] == 40


# ---------------------------------------------------------------- walls (md-ref/tests/boundaries.rs)
def _gas_in_walls(O, n, density, aspect, seed):
    """boundaries.rs:6-10: a WCA gas between hard walls on y (the lattice clear of them)."""
    from micrographia_gb300 import Wall

    sys_ = System(box_for(n, density, aspect), 0.005, Pair.wca(), [1.0]).with_walls(1, Wall.hard(), Wall.hard())
    return sys_, O.fluid(sys_, n, 1.0, seed)


@pytest.mark.parametrize("kind", ["hard", "soft"])
def test_oracle_walls_and_gravity_reverse_exactly(O, kind):
    """boundaries.rs:12-35: hard (soft) walls on both axes with gravity; 2000 steps, reverse,
    2000 steps, reverse: the initial state exactly; the walls were hit (pushed)."""
    from micrographia_gb300 import Wall

    sys_, s0 = _gas_in_walls(O, 400, 0.3, 1.0, 1)
    w = Wall.hard() if kind == "hard" else Wall.soft()
    sys_.with_walls(0, w, w).with_gravity([0.0, -0.5])
    if kind == "soft":
        sys_.with_walls(1, w, w)
    e = O.IntEngine(sys_, s0)
    e.step(2000)
    energy, impulse, hits = e.wall_ledger()
    if kind == "hard":
        assert sum(hits) > 100
    else:
        assert sum(impulse) > 1.0
    e.reverse()
    e.step(2000)
    e.reverse()
    assert e.state == s0


def test_oracle_energy_with_gravity_and_soft_walls_is_conserved(O):
    """boundaries.rs:37-54: a stratified gas (m g H / T = 2) between soft walls, f64 engine:
    total energy per particle within 2e-3 over 2000 steps."""
    from micrographia_gb300 import Wall

    sys_, s0 = _gas_in_walls(O, 400, 0.3, 1.0, 2)
    g = 2.0 / sys_.box_f64()[1]
    sys_.with_walls(1, Wall.soft(), Wall.soft()).with_gravity([0.0, -g])
    e = O.IntEngine(sys_, s0, f64=True)
    e.step(200)
    e0 = sum(e.energy())
    worst = 0.0
    for _ in range(20):
        e.step(100)
        worst = max(worst, abs(sum(e.energy()) - e0) / 400)
    assert worst < 2e-3


def _thermal_velocity_py(sys_, i, clock, t, m, inward, dim):
    """walls::thermal_velocity (walls.rs:89-101) / three::thermal_velocity (three.rs:222-243)."""
    from micrographia_gb300.workloads import threefry2x32

    k0, k1 = sys_.seed & 0xFFFFFFFF, ((sys_.seed >> 32) ^ 0x57414C4C) & 0xFFFFFFFF
    full = lambda r: (((r[0] << 21) ^ (r[1] >> 11)) & ((1 << 53) - 1)) * (1.0 / (1 << 53))
    unit = lambda w: ((w << 21) & ((1 << 53) - 1)) * (1.0 / (1 << 53))
    r = threefry2x32(i, clock, k0, k1)
    r2 = threefry2x32(i, clock, k0, k1 ^ 1)
    u1, u2, u3 = 1.0 - full(r), 1.0 - unit(r2[0]), unit(r2[1])
    sd = math.sqrt(t / m)
    normal = inward * sd * math.sqrt(-2.0 * math.log(u1))
    if dim == 2:
        return normal, [sd * math.sqrt(-2.0 * math.log(u2)) * math.cos(2.0 * math.pi * u3)]
    rad = sd * math.sqrt(-2.0 * math.log(u2))
    a = 2.0 * math.pi * u3
    return normal, [rad * math.cos(a), rad * math.sin(a)]


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_wall_collisions_match_a_python_restatement(O, dim):
    """Particles that never interact (a 0.1-sigma pair), moving at 0.25 sigma per step between a
    hot thermal wall, a cold thermal wall and (3D) hard walls: every step the oracle's mirror and
    collide (int_engine.rs:316-330, 363-390; int_engine3.rs:186-205) equal a Python restatement,
    and the ledger's energy, impulse and hits equal the same sums in the same order."""
    from micrographia_gb300 import State, State3, System3 as S3, Wall

    L, n = 12.0, 6
    tiny = Pair(1.0, 0.1, 0.1 * 2 ** (1 / 6))
    box = [int(L * ONE)] * dim
    wall_axis = 0
    hot, cold = Wall.thermal(2.0), Wall.thermal(0.5)
    if dim == 2:
        sys_ = System(box, 0.005, tiny, [1.0, 3.0]).with_walls(0, hot, cold)
    else:
        sys_ = S3(box, 0.005, tiny, [1.0, 3.0]).with_walls(0, hot, cold).with_walls(2, Wall.hard(), Wall.hard())
    sys_.seed = 0x2468_ACE0_1357
    rng = np.random.default_rng(5)
    pos = (rng.random((n, dim)) * (L - 2) + 1) * ONE
    pos = pos.astype(np.int64)
    vel = (rng.choice([-1, 1], (n, dim)) * rng.uniform(0.05, 0.25, (n, dim)) * ONE).astype(np.int32)
    sp = np.array([k % 2 for k in range(n)], np.uint32)
    st = (State if dim == 2 else State3)(pos, vel, sp)
    c = O.IntEngine(sys_, st)
    led_e, led_p, led_h = [0.0] * 7, [0.0] * 7, [0] * 7
    lbox = box[0]
    vfl = lambda v: float(v) / 2**32 / sys_.dt
    for clock in range(300):
        before = c.state
        c.step(1)
        after = c.state
        for i in range(n):
            x = [int(v) for v in before.pos[i]]
            v = [int(u) for u in before.vel[i]]
            x = [x[a] + v[a] for a in range(dim)]
            for a in range(dim):
                if sys_.periodic(a):
                    x[a] %= lbox
                    continue
                side = 0 if x[a] < 0 else (1 if x[a] >= lbox else None)
                if side is None:
                    continue
                x[a] = -1 - x[a] if side == 0 else 2 * lbox - 1 - x[a]
                m = sys_.masses[int(sp[i])]
                b = [vfl(u) for u in v]
                w = sys_.walls[a][side]
                if w.kind == 3:
                    vn, vt = _thermal_velocity_py(sys_, i, clock, w.t, m, 1.0 if side == 0 else -1.0, dim)
                    v[a] = sys_.to_step_displacement(vn)
                    others = [1 - a] if dim == 2 else [(a + 1) % 3, (a + 2) % 3]
                    for o, t in zip(others, vt):
                        v[o] = sys_.to_step_displacement(t)
                else:
                    v[a] = -v[a]
                af = [vfl(u) for u in v]
                ke = lambda u: 0.5 * m * sum(q * q for q in u) if dim == 3 else 0.5 * m * (u[0] * u[0] + u[1] * u[1])
                slot = 2 * a + side
                led_e[slot] += ke(af) - ke(b)
                led_p[slot] += abs(m * (b[a] - af[a]))
                led_h[slot] += 1
            assert list(after.pos[i]) == x and list(after.vel[i]) == v, (clock, i)
    e_, p_, h_ = c.wall_ledger()
    assert h_ == led_h and h_[0] > 0 and h_[1] > 0
    assert e_ == led_e and p_ == led_p


def _on_step_temperatures(sys_, e):
    """IntEngine::velocities (int_engine.rs:417-430), for systems without gravity: per particle
    0.5 m |(v + v_next) / 2|^2 with v_next = v + kick."""
    k, _ = e.kicks()
    st = e.state
    v0 = st.vel.astype(np.float64) / 2**32 / sys_.dt
    v1 = (st.vel.astype(np.int64) + k).astype(np.float64) / 2**32 / sys_.dt
    v = 0.5 * (v0 + v1)
    m = np.array(sys_.masses)[st.species]
    return 0.5 * m * (v * v).sum(axis=1), st.species


def test_oracle_thermal_walls_set_the_temperature(O):
    """boundaries.rs:91-110: a dilute WCA gas at T = 0.5 between thermal walls at 1.5 reaches
    T = 1.5 within 0.06, taking more than 0.5 epsilon per particle from the walls."""
    from micrographia_gb300 import Wall

    n = 150
    w = Wall.thermal(1.5)
    sys_ = System(box_for(n, 0.1, 1.0), 0.005, Pair.wca(), [1.0]).with_walls(0, w, w).with_walls(1, w, w)
    e = O.IntEngine(sys_, O.fluid(sys_, n, 0.5, 4))
    e.step(40000)
    t = 0.0
    for _ in range(200):
        e.step(100)
        ke, _ = _on_step_temperatures(sys_, e)
        t += ke.sum() / n / 200
    heat = sum(e.wall_ledger()[0])
    assert abs(t - 1.5) < 0.06, t
    assert heat > 0.5 * n


def test_oracle_andersen_sets_the_temperature_of_each_species(O):
    """boundaries.rs:217-239: an LJ liquid of masses 1 and 4 from T = 2 under a bath at 0.8
    (rate 1): each species' on-step temperature within 0.04 of 0.8."""
    n = 800
    sys_ = System(box_for(n, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0, 4.0]).with_thermostat(0.8, 1.0)
    s0 = O.fluid(sys_, n, 2.0, 11)
    s0.species[0::2] = 1
    e = O.IntEngine(sys_, s0)
    e.step(3000)
    t = np.zeros(2)
    for _ in range(40):
        e.step(50)
        ke, sp = _on_step_temperatures(sys_, e)
        for s in (0, 1):
            t[s] += ke[sp == s].sum() / (n / 2) / 40
    assert abs(t[0] - 0.8) < 0.04 and abs(t[1] - 0.8) < 0.04, t


def test_oracle_membrane_confines_solute_and_is_reversible(O):
    """md-ref/tests/boundaries.rs:241-268: soft walls on x, a membrane at the middle blocking
    species 1 (the solute, 20% of the right half): after 3000 steps no solute has crossed, the
    solute has hit the membrane, the solvent has crossed it, and the run reverses exactly."""
    from micrographia_gb300 import Wall
    from micrographia_gb300.workloads import uniform

    n = 1200
    sys_ = System(box_for(n, 0.4, 2.0), 0.005, Pair.wca(), [1.0, 1.0]).with_walls(0, Wall.soft(), Wall.soft())
    half = sys_.box_f64()[0] / 2.0
    sys_.with_membrane(0, half, [1])
    s0 = O.fluid(sys_, n, 1.0, 13)
    for i in range(n):
        if to_f64(int(s0.pos[i, 0])) > half + 1.0 and uniform(13, 3, i) < 0.2:
            s0.species[i] = 1
    left0 = int((s0.pos[:, 0] < int(half * ONE)).sum())
    e = O.IntEngine(sys_, s0)
    e.step(3000)
    st = e.state
    assert all(to_f64(int(p)) > half - 0.5 for p in st.pos[st.species == 1, 0])
    assert e.wall_ledger()[2][5] > 20
    assert int((st.pos[:, 0] < int(half * ONE)).sum()) != left0
    e.reverse()
    e.step(3000)
    e.reverse()
    assert e.state == s0


def _compartment_fluid(O, sys_, per_box, t, seed):
    """init::compartment_fluid (init.rs:126-149): per_box particles on a small jittered lattice
    in every compartment, 0.6 sigma clear of its walls, numbered box by box; Maxwell velocities."""
    from micrographia_gb300 import State, to_fixed
    from micrographia_gb300.workloads import uniform

    cx, cy = sys_.compartment_counts()
    side = [to_f64(sys_.box_len[0]) / cx, to_f64(sys_.box_len[1]) / cy]
    nx = max(int(math.ceil(math.sqrt(per_box * side[0] / side[1]))), 1)
    ny = -(-per_box // nx)
    margin = 0.6
    a = [(side[0] - 2.0 * margin) / nx, (side[1] - 2.0 * margin) / ny]
    pos = []
    for by in range(cy):
        for bx in range(cx):
            for k in range(per_box):
                i = len(pos)
                jx = 0.2 * a[0] * (uniform(seed, 2, 2 * i) - 0.5)
                jy = 0.2 * a[1] * (uniform(seed, 2, 2 * i + 1) - 0.5)
                x = bx * side[0] + margin + ((k % nx) + 0.5) * a[0] + jx
                y = by * side[1] + margin + ((k // nx) + 0.5) * a[1] + jy
                pos.append([to_fixed(x), to_fixed(y)])
    n = len(pos)
    sp = np.zeros(n, np.uint32)
    return State(np.array(pos, np.int64), O.maxwell(sys_, sp, t, seed), sp)


def test_oracle_compartments_are_independent_and_reversible(O):
    """md-ref/tests/boundaries.rs:154-181: 16 x 16 compartments of 8 sigma between hard walls,
    6 particles each: after 3000 steps every particle is still in its own compartment, and the run
    reverses exactly."""
    from micrographia_gb300 import Wall

    side = 8 * ONE
    sys_ = System([16 * side, 16 * side], 0.005, Pair.wca(), [1.0])
    sys_.with_walls(0, Wall.hard(), Wall.hard()).with_walls(1, Wall.hard(), Wall.hard())
    sys_.with_compartments(0, 3).with_compartments(1, 3)
    s0 = _compartment_fluid(O, sys_, 6, 1.0, 7)
    home = [sys_.compartment_of(p) for p in s0.pos]
    e = O.IntEngine(sys_, s0)
    e.step(3000)
    assert [sys_.compartment_of(p) for p in e.state.pos] == home
    e.reverse()
    e.step(3000)
    e.reverse()
    assert e.state == s0


# ---------------------------------------------------------------- bonds (md-ref/tests/polymers.rs)
def _melt(O, n_chains, length, density, seed):
    """polymers.rs:6-14: Kremer-Grest chains (FENE k = 30, R0 = 1.5, WCA beads) laid out
    straight (init::chains, bond 0.97 sigma), Maxwell velocities at T = 1."""
    from micrographia_gb300 import Bond, chains

    n = n_chains * length
    sys_ = System(box_for(n, density, 1.0), 0.005, Pair.wca(), [1.0])
    pos, bonds = chains(sys_, n_chains, length, 0.97)
    sys_.with_bonds([Bond.kremer_grest()], bonds)
    sp = np.zeros(n, np.uint32)
    return sys_, State(pos, O.maxwell(sys_, sp, 1.0, seed), sp)


def test_oracle_chains_are_exactly_reversible(O):
    """polymers.rs:17-25: 20 chains of 20 beads at density 0.3, IntEngine<f32>: 2000 steps,
    reverse, 2000 steps, reverse: the initial state exactly."""
    sys_, s0 = _melt(O, 20, 20, 0.3, 1)
    e = O.IntEngine(sys_, s0)
    e.step(2000)
    assert e.state != s0
    e.reverse()
    e.step(2000)
    e.reverse()
    assert e.state == s0


def test_oracle_chains_hold_together_and_conserve_energy(O):
    """polymers.rs:28-50: the f64 engine's energy per bead within 2e-3 over 2000 steps after 500,
    and the mean bond length within 0.03 of the Kremer-Grest 0.97 sigma."""
    sys_, s0 = _melt(O, 20, 20, 0.3, 2)
    e = O.IntEngine(sys_, s0, f64=True)
    e.step(500)
    e0 = sum(e.energy())
    worst = 0.0
    for _ in range(10):
        e.step(200)
        worst = max(worst, abs(sum(e.energy()) - e0) / 400.0)
    st = e.state
    box = np.array(sys_.box_len, np.int64)
    lengths = []
    for a, b, _ in sys_.bonds:
        d = st.pos[b] - st.pos[a]
        d = np.where(d >= box // 2, d - box, np.where(d < -(box // 2), d + box, d))
        lengths.append(math.hypot(*(d / 2**32)))
    assert worst < 2e-3, worst
    assert abs(np.mean(lengths) - 0.97) < 0.03, np.mean(lengths)


def test_oracle_bond_kicks_match_a_python_restatement(O):
    """A harmonic bond (k = 50, r0 = 1), a zero-length tether and a FENE bond stretched past its
    0.999999 cap, between non-interacting particles: the oracle's kicks equal BondConsts::eval
    (real.rs:175-196) and the rounding of IntEngine::forces (int_engine.rs:185-202) restated in
    numpy f32, and Newton's third law holds exactly."""
    from micrographia_gb300 import Bond

    tiny = Pair(1.0, 0.1, 0.1 * 2 ** (1 / 6))
    sys_ = System([int(40 * ONE), int(40 * ONE)], 0.005, tiny, [1.0, 2.0])
    types = [Bond.harmonic(50.0, 1.0), Bond.harmonic(3.0, 0.0), Bond.fene_bond(30.0, 1.5)]
    pos = np.array([[5, 5], [6.3, 5.4], [20, 20], [20.7, 21.1], [30, 30], [31.6, 30.05], [2, 2], [38.5, 39.2]], np.float64)
    pos = (pos * ONE).astype(np.int64)
    bonds = [(0, 1, 0), (2, 3, 1), (4, 5, 2), (6, 7, 0)]  # the last across the periodic boundary
    sys_.with_bonds(types, bonds)
    sp = np.array([0, 1, 0, 1, 0, 1, 1, 0], np.uint32)
    st = State(pos, np.zeros((8, 2), np.int32), sp)
    k, _ = O.IntEngine(sys_, st).kicks()
    f32 = np.float32
    box = np.array(sys_.box_len, np.int64)
    for a, b, t in bonds:
        assert (k[a].astype(np.int64) + k[b] == 0).all() or sys_.masses[sp[a]] != sys_.masses[sp[b]]
        for i, j in ((a, b), (b, a)):
            d = pos[j] - pos[i]
            d = np.where(d >= box // 2, d - box, np.where(d < -(box // 2), d + box, d))
            f = [f32(O.sep_f32(int(x))) for x in d]
            r2 = f32(f[0] * f[0]) + f32(f[1] * f[1])
            bt = types[t]
            kk, r0 = f32(bt.k), f32(bt.r0)
            if bt.fene:
                x = min(f32(r2 / f32(r0 * r0)), f32(0.999999))
                fr = f32(-kk / f32(f32(1) - x))
            elif r0 == 0:
                fr = -kk
            else:
                r = f32(np.sqrt(r2))
                fr = f32(f32(-kk * f32(r - r0)) / r)
            c = f32(sys_.dt * sys_.dt / sys_.masses[sp[i]] * 2**32)
            aa = f32(-fr * c)
            # round half to even, saturating like Rust's `as i32` (the stretched FENE bond saturates)
            want = [int(min(max(np.rint(f32(aa * fa)), -(2**31)), 2**31 - 1)) for fa in f]
            assert list(k[i]) == want, (i, j, t)


# ---------------------------------------------------------------- pistons (md-ref/tests/boundaries.rs:270-338)
def _gas_under_piston(O, n, density, drive, seed):
    """boundaries.rs:270-285: a WCA gas in a box twice the height of box_for's, soft floor, hard
    roof, the piston starting at half the height (stopping at 2 sigma); the fluid lattice
    squeezed into the lower half."""
    from micrographia_gb300 import Wall

    bl = box_for(n, density, 1.0)
    bl[1] *= 2
    h = to_f64(bl[1]) / 2.0
    sys_ = System(bl, 0.005, Pair.wca(), [1.0]).with_walls(1, Wall.soft(), Wall.hard()).with_piston(drive, h, 2.0)
    s = O.fluid(sys_, n, 1.0, seed)
    s.pos[:, 1] //= 2
    return sys_, s


def test_oracle_moving_piston_is_exactly_reversible(O):
    """boundaries.rs:287-298: 500 particles under a piston driven down at 0.5 sigma/tau: 2000 steps
    lower it; reversed, 2000 steps and reversed again, the state and the piston's height exactly."""
    from micrographia_gb300 import Piston

    sys_, s0 = _gas_under_piston(O, 500, 0.3, Piston.speed_drive(-0.5), 16)
    e = O.IntEngine(sys_, s0)
    w0 = e.piston()[0]
    e.step(2000)
    assert e.piston()[0] < w0
    e.reverse()
    e.step(2000)
    e.reverse()
    assert e.state == s0
    assert e.piston()[0] == w0


def test_oracle_free_piston_balances_the_pressure(O):
    """boundaries.rs:300-319: a free piston (mass 50, 15 eps/sigma pushing down) over 600 particles
    settles where the time-averaged pressure on the floor (its ledger impulse over 60,000 steps
    after 10,000) equals the piston's external pressure within 5%."""
    from micrographia_gb300 import Piston

    force = 15.0
    sys_, s0 = _gas_under_piston(O, 600, 0.2, Piston.free(50.0, force), 17)
    width = sys_.box_f64()[0]
    e = O.IntEngine(sys_, s0)
    e.step(10000)
    before = e.wall_ledger()[1][2]
    steps = 60000
    e.step(steps)
    p_bottom = (e.wall_ledger()[1][2] - before) / (steps * sys_.dt * width)
    assert abs(p_bottom / (force / width) - 1.0) < 0.05, p_bottom


def test_oracle_fast_compression_heats_more_than_adiabatic(O):
    """boundaries.rs:321-338: 400 particles (density 0.05) compressed to a third of the height at
    0.4 sigma/tau by IntEngine<f64>: T A grows by more than 5% (slow compression keeps T A, the 2D
    adiabat), and the work the piston did is the energy the gas gained, within 1%."""
    from micrographia_gb300 import Piston

    n = 400
    sys_, s0 = _gas_under_piston(O, n, 0.05, Piston.speed_drive(-0.4), 18)
    width = sys_.box_f64()[0]
    e = O.IntEngine(sys_, s0, f64=True)
    t0, h0 = e.energy()[0] / n, to_f64(e.piston()[0])
    k0 = sum(e.energy())
    steps = int((h0 * 2.0 / 3.0) / (0.4 * sys_.dt))
    e.step(steps)
    t1, h1 = e.energy()[0] / n, to_f64(e.piston()[0])
    a0, a1 = width * (h0 - 1.0), width * (h1 - 1.0)
    assert t1 * a1 > 1.05 * t0 * a0, (t0 * a0, t1 * a1)
    gained = sum(e.energy()) - k0
    assert abs(gained + e.piston()[2]) < 0.01 * gained, (gained, e.piston()[2])


def test_fdlibm_and_the_platform_libm_on_bath_draws(O):
    """The device's heat bath computes ln, cos and sin with fdlibm (as the reference's wasm build
    does); the reference's native build calls the platform libm, and so does the oracle. Over
    2 x 10^7 of the bath's own draws (kT/m = 1, dt = 0.005) this counts how often the two round
    differently and whether that ever changes a redrawn velocity: a step displacement (~2^24 units
    here) changes only when the f64 velocity lies within its last bit (~2^-28 units) of a rounding
    edge, about 4e-9 of the draws whose ln, cos or sin differ, so none is expected."""
    n = 20_000_000
    d_log, d_cos, d_sin, flips = O.libm_compare(n, 0x5EED_1234, 1.0, 0.005)
    print(f"ln {d_log / n:.2e}, cos {d_cos / n:.2e}, sin {d_sin / n:.2e} of draws rounded differently; {flips} velocity changes")
    assert flips == 0
    assert max(d_log, d_cos, d_sin) < n // 10  # (measured: ln 7%, cos and sin 3% of draws, last bit)


def test_half_shell_3d_equals_the_reference_loop(O):
    """The CPU baseline's half-shell 3D loop (each pair once, each side rounded on its own) gives
    IntEngine3's kicks bit for bit, and the same 40-step trajectory: one species, and a mixture
    with two masses, an unlike pair and a pair 0.3 sigma apart whose kicks saturate."""
    from micrographia_gb300 import ONE, Pair, System3, cube_for

    for masses in ([1.0], [1.0, 2.5]):
        n = 2048
        sys3 = System3(cube_for(n, 0.8442), 0.005, Pair.lj(2.5), masses)
        if len(masses) == 2:
            sys3.with_pair(0, 1, Pair(0.7, 1.05, 2.5))
        s0 = O.fcc_maxwell(sys3, n, 0.72, 3, jitter=0.05)
        if len(masses) == 2:
            s0.species[::3] = 1
            s0.pos[1] = s0.pos[0] + np.array([int(0.3 * ONE), 0, 0])
        a = O.IntEngine(sys3, s0, threads=2)
        b = O.IntEngine(sys3, s0, threads=2, half3=True)
        ka, pa = a.kicks()
        kb, pb = b.kicks()
        assert np.array_equal(ka, kb)
        assert abs(pa - pb) < 1e-6 * abs(pa)
        if len(masses) == 2:
            assert np.abs(ka[:2, 0].astype(np.int64)).min() > 2**30  # the saturated pair dominates
        if len(masses) == 1:
            a.step(40)
            b.step(40)
            assert a.state == b.state
