"""The force kernel's scenario epilogue: with one force lane per particle (every system of at least
262,144 particles, every multi-species system, or GBMD_FLAG_FORCE_LANES(1)) the Verlet-list force
kernel adds the bonds', soft walls' and piston's kicks to the pair kicks and runs the bath, the
membrane, the walls' mirrors and collisions and the piston's mirror after its leapfrog, instead of
the separate passes that split force lanes use. Both forms are checked here against the oracle,
bit for bit, with the ledger and the piston's state, on the scenarios of the wall, bond and
piston tests."""

import numpy as np
import pytest

from micrographia_gb300 import ForceMode, GpuEngine, GpuEngine3, Pair, Piston, System, System3, Wall, _abi, box_for, cube_for
from test_gpu_walls import _gas_in_walls, _same_ledger

pytestmark = pytest.mark.gpu

LANES = [pytest.param(1, id="epilogue"), pytest.param(2, id="passes")]


def _run_both(O, sys_, s0, steps, lanes, reverse=False, engine=GpuEngine):
    c = O.IntEngine(sys_, s0)
    with engine(sys_, s0, ForceMode.verlet_with_skin(sys_, s0.n(), 0.3), flags=_abi.force_lanes_flag(lanes)) as g:
        g.step(steps)
        c.step(steps)
        assert g.read_state() == c.state
        _same_ledger(g, c)
        if getattr(sys_, "piston", None):
            assert g.piston() == c.piston()[:3]
        kg, _ = g.kicks()
        kc, _ = c.kicks()
        assert np.array_equal(kg, kc)
        if reverse:
            g.reverse()
            g.step(steps)
            g.reverse()
            assert g.read_state() == s0


@pytest.mark.parametrize("lanes", LANES)
@pytest.mark.parametrize("kind", ["hard", "soft"])
def test_walls_with_gravity(O, kind, lanes):
    sys_, s0 = _gas_in_walls(O, 400, 0.3, 1, kind, 0.5)
    _run_both(O, sys_, s0, 1500, lanes, reverse=True)


@pytest.mark.parametrize("lanes", LANES)
def test_kremer_grest_melt_between_walls(O, lanes):
    from test_gpu_bonds import _melt

    sys_, s0 = _melt(O, 20, 20, 0.3, 3, walls=True)
    _run_both(O, sys_, s0, 1500, lanes, reverse=True)


@pytest.mark.parametrize("lanes", LANES)
def test_driven_piston_with_a_bath(O, lanes):
    from test_oracle import _gas_under_piston

    sys_, s0 = _gas_under_piston(O, 400, 0.3, Piston.speed_drive(0.3), 19)
    sys_.with_thermostat(1.2, 2.0)
    _run_both(O, sys_, s0, 1500, lanes)


@pytest.mark.parametrize("lanes", LANES)
def test_free_piston(O, lanes):
    from test_oracle import _gas_under_piston

    sys_, s0 = _gas_under_piston(O, 600, 0.2, Piston.free(50.0, 15.0), 17)
    _run_both(O, sys_, s0, 2000, lanes)


@pytest.mark.parametrize("lanes", LANES)
def test_membrane_with_pores_and_thermal_walls(O, lanes):
    """Thermal walls on x (hot and cold) and a membrane with pores blocking the solute."""
    from micrographia_gb300 import to_f64
    from micrographia_gb300.workloads import uniform

    n = 1200
    sys_ = System(box_for(n, 0.4, 2.0), 0.005, Pair.wca(), [1.0, 1.0]).with_walls(0, Wall.thermal(1.5), Wall.thermal(0.8))
    half = sys_.box_f64()[0] / 2.0
    sys_.with_membrane(0, half, [1]).with_pores(1, 0.5)
    s0 = O.fluid(sys_, n, 1.0, 13)
    for i in range(n):
        if to_f64(int(s0.pos[i, 0])) > half + 1.0 and uniform(13, 3, i) < 0.2:
            s0.species[i] = 1
    _run_both(O, sys_, s0, 2000, lanes)


@pytest.mark.parametrize("lanes", LANES)
def test_compartments(O, lanes):
    from micrographia_gb300 import ONE
    from test_oracle import _compartment_fluid

    side = 8 * ONE
    sys_ = System([16 * side, 16 * side], 0.005, Pair.wca(), [1.0])
    sys_.with_walls(0, Wall.hard(), Wall.hard()).with_walls(1, Wall.hard(), Wall.hard())
    sys_.with_compartments(0, 3).with_compartments(1, 3)
    s0 = _compartment_fluid(O, sys_, 6, 1.0, 7)
    _run_both(O, sys_, s0, 1500, lanes, reverse=True)


@pytest.mark.parametrize("lanes", LANES)
def test_walled_liquid_3d_with_a_bath(O, lanes):
    """3D: soft walls on z, thermal walls on x, a bath on species 0."""
    n = 4000
    sys3 = System3(cube_for(n, 0.6), 0.005, Pair.lj(2.5), [1.0])
    sys3.with_walls(2, Wall.soft(), Wall.soft()).with_walls(0, Wall.thermal(1.0), Wall.thermal(0.6))
    sys3.with_thermostat(0.9, 1.0)
    s0 = O.fcc_maxwell(sys3, n, 0.9, 5, jitter=0.05)
    L = sys3.box_len
    from micrographia_gb300 import ONE

    for a in (0, 2):  # a sigma clear of the walls
        s0.pos[:, a] = (ONE + s0.pos[:, a].astype(np.float64) / L[a] * (L[a] - 2 * ONE)).astype(np.int64)
    _run_both(O, sys3, s0, 600, lanes, engine=GpuEngine3)
