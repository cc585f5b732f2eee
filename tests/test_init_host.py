"""md-core's init helpers in the package (micrographia_gb300.init) against the oracle: the
host-side ones here (no GPU), the device-side ones under the gpu mark."""

import numpy as np
import pytest

from micrographia_gb300 import ONE, Pair, State, State3, System, System3, box_for, cube_for, init


def _vel(rng, n, d):
    return rng.integers(-(2**24), 2**24, (n, d)).astype(np.int32)


@pytest.mark.parametrize("dim", [2, 3])
def test_zero_sum_temperature_and_kinetic_equal_the_oracle(O, dim):
    """zero_velocity_sum, half_step_kinetic and set_temperature (init.rs:76-103, three.rs:299-308,
    376-404) on random velocities with two masses (3D: species 2 pinned): bit for bit."""
    rng = np.random.default_rng(dim)
    n = 5001
    if dim == 2:
        sys_ = System(box_for(n, 0.5, 1.0), 0.005, Pair.lj(2.5), [1.0, 2.0, 0.7])
        S = State
    else:
        sys_ = System3(cube_for(n, 0.5), 0.005, Pair.lj(2.5), [1.0, 2.0, 0.7]).with_pinned(2)
        S = State3
    sp = (rng.integers(0, 3, n)).astype(np.uint32)
    st = S(np.zeros((n, dim), np.int64), _vel(rng, n, dim), sp)
    assert init.half_step_kinetic(sys_, st) == O.half_step_kinetic(sys_, st)
    want = O.set_temperature(sys_, st, 0.8)
    got = init.set_temperature(st.copy(), sys_, 0.8).vel
    assert np.array_equal(got, want)
    v = _vel(rng, n, dim)
    w = v.copy()
    O.lib().oracle_zero_velocity_sum(C_sys(sys_), sp.ctypes.data_as(O.U32P), n, w.ctypes.data_as(O.I32P))
    init.zero_velocity_sum(v, sys_, sp)
    assert np.array_equal(v, w)


def C_sys(sys_):
    import ctypes as C

    c = sys_.to_c()
    C_sys.keep = c
    return C.byref(c)


def test_mark_disc_equals_the_oracle(O):
    """mark_disc (init.rs:152-163) with a disc across the periodic boundary and particles on its
    rim."""
    rng = np.random.default_rng(4)
    n = 4000
    sys_ = System(box_for(n, 0.5, 1.5), 0.005, Pair.lj(2.5), [1.0, 1.0])
    pos = np.stack([rng.integers(0, sys_.box_len[0], n), rng.integers(0, sys_.box_len[1], n)], axis=1).astype(np.int64)
    pos[0] = [int(1.0 * ONE), int(3.0 * ONE)]  # exactly at the radius from (1, 8): not inside
    st = State(pos, np.zeros((n, 2), np.int32), np.zeros(n, np.uint32))
    want = O.mark_disc(sys_, st, [1.0, 8.0], 5.0, 1)
    got = init.mark_disc(st.copy(), sys_, [1.0, 8.0], 5.0, 1).species
    assert np.array_equal(got, want)
    assert 0 < got.sum() < n and got[0] == 0


def test_barometric_positions_equal_the_oracle(O):
    """barometric's draws and rejections (init.rs:223-260): two species under gravity, a column
    dense enough that many draws are rejected."""
    sys_ = System([int(20 * ONE), int(40 * ONE)], 0.005, Pair.wca(), [1.0, 3.0]).with_gravity([0.0, -0.05])
    sp = (np.arange(300) % 2).astype(np.uint32)
    got = init.barometric_positions(sys_, sp, 1.0, 0.9, 1.1, 5)
    want = O.barometric_positions(sys_, sp, 1.0, 0.9, 1.1, 5)
    assert np.array_equal(got, want)
    assert got[:, 1].min() >= int(1.1 * ONE) - 1 and got[:, 1].max() <= sys_.box_len[1] - int(1.1 * ONE) + 1


@pytest.mark.gpu
def test_device_side_init_helpers_equal_the_oracle(O):
    """fixed_speed (init.rs:61-74, fdlibm cos/sin on the device), lattice (init.rs:22-38),
    compartment_fluid (init.rs:126-149) and barometric's velocities, against the oracle."""
    from test_oracle import _compartment_fluid

    n = 3001
    sys_ = System(box_for(n, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0, 2.0])
    sp = (np.arange(n) % 2).astype(np.uint32)
    assert np.array_equal(init.fixed_speed(sys_, sp, 1.3, 9), O.fixed_speed(sys_, sp, 1.3, 9))
    want = np.empty((n, 2), np.int64)
    import ctypes as C

    box = (C.c_int64 * 2)(*sys_.box_len[:2])
    O.lib().oracle_lattice(n, box, 0.1, 17, want.ctypes.data_as(O.I64P))
    assert np.array_equal(init.lattice(n, sys_.box_len, 0.1, 17), want)
    from micrographia_gb300 import Wall

    sc = System([int(64 * ONE), int(64 * ONE)], 0.005, Pair.wca(), [1.0])
    sc.with_walls(0, Wall.hard(), Wall.hard()).with_walls(1, Wall.hard(), Wall.hard())
    sc.with_compartments(0, 3).with_compartments(1, 3)
    assert init.compartment_fluid(sc, 6, 1.0, 7) == _compartment_fluid(O, sc, 6, 1.0, 7)
    sb = System([int(20 * ONE), int(40 * ONE)], 0.005, Pair.wca(), [1.0, 3.0]).with_gravity([0.0, -0.05])
    spb = (np.arange(200) % 2).astype(np.uint32)
    got = init.barometric(sb, spb, 1.0, 0.9, 1.1, 5)
    assert np.array_equal(got.pos, O.barometric_positions(sb, spb, 1.0, 0.9, 1.1, 5))
    assert np.array_equal(got.vel, O.maxwell(sb, spb, 1.0, 5))
