"""Bonds on the GPU engine (2D; md_core::BondType, system.rs:70-96; IntEngine::forces,
int_engine.rs:185-202), against the oracle's IntEngine<f32> bit for bit.

Scenarios from the reference's own tests: Kremer-Grest chains (crates/md-ref/tests/polymers.rs:
6-25, exact reversal), harmonic dimers in an LJ solvent (crates/md-ref/tests/fast_path.rs:48-53),
and bonds stretched past the FENE cap, zero-length tethers and bonds across the periodic
boundary."""

import numpy as np
import pytest

from micrographia_gb300 import ONE, Bond, ForceMode, GpuEngine, GpuEngine3, Pair, State, System, System3, Wall, box_for, chains, cube_for

pytestmark = pytest.mark.gpu


def _melt(O, n_chains, length, density, seed, walls=False):
    n = n_chains * length
    sys_ = System(box_for(n, density, 1.0), 0.005, Pair.wca(), [1.0])
    if walls:
        sys_.with_walls(1, Wall.soft(), Wall.soft())
    pos, bonds = chains(sys_, n_chains, length, 0.97)
    sys_.with_bonds([Bond.kremer_grest()], bonds)
    sp = np.zeros(n, np.uint32)
    return sys_, State(pos, O.maxwell(sys_, sp, 1.0, seed), sp)


@pytest.mark.parametrize("mode", ["cells", "verlet"])
def test_chains_follow_the_oracle_and_reverse(O, mode):
    """polymers.rs:17-25 on the GPU: 20 chains of 20 beads at density 0.3: 2000 steps equal
    IntEngine<f32>'s bit for bit (kicks too), and reversed they return exactly."""
    sys_, s0 = _melt(O, 20, 20, 0.3, 1)
    n = s0.n()
    m = ForceMode.cell_list() if mode == "cells" else ForceMode.verlet_with_skin(sys_, n, 0.3)
    c = O.IntEngine(sys_, s0)
    with GpuEngine(sys_, s0, m) as g:
        g.step(2000)
        c.step(2000)
        assert g.read_state() == c.state
        kg, peg = g.kicks()
        kc, pec = c.kicks()
        assert np.array_equal(kg, kc)
        assert abs(peg - pec) <= 1e-5 * abs(pec)
        g.reverse()
        g.step(2000)
        g.reverse()
        assert g.read_state() == s0


def test_chains_between_soft_walls_follow_the_oracle(O):
    """The same melt between soft walls on y: bonds, walls and their ledger together."""
    sys_, s0 = _melt(O, 20, 20, 0.3, 3, walls=True)
    c = O.IntEngine(sys_, s0)
    with GpuEngine(sys_, s0, ForceMode.verlet_with_skin(sys_, s0.n(), 0.3)) as g:
        g.step(1500)
        c.step(1500)
        assert g.read_state() == c.state
        ge, gp, gh = g.read_ledger()
        oe, op = c.wall_ledger_fixed()
        assert [round(x * 2**24) for x in gp] == list(op)


@pytest.mark.parametrize("mode", ["cells", "verlet"])
def test_bonded_pairs_in_an_lj_solvent_follow_the_oracle(O, mode):
    """fast_path.rs:48-53: a fluid of 1200 LJ particles (rho 0.5, T 1) in which ids 2k, 2k + 1
    (k < 200) are joined by harmonic bonds (k = 50, r0 = 1) wherever they stand, so the pairs
    swing across the box at up to a sigma per step: 300 steps equal IntEngine<f32>'s bit for bit,
    and the potentials agree within 1e-4 relative."""
    n = 1200
    sys_ = System(box_for(n, 0.5, 1.0), 0.005, Pair.lj(2.5), [1.0])
    s0 = O.fluid(sys_, n, 1.0, 3)
    sys_.with_bonds([Bond.harmonic(50.0, 1.0)], [(2 * k, 2 * k + 1, 0) for k in range(200)])
    m = ForceMode.cell_list() if mode == "cells" else ForceMode.verlet_with_skin(sys_, n, 0.3)
    c = O.IntEngine(sys_, s0)
    with GpuEngine(sys_, s0, m) as g:
        g.step(300)
        c.step(300)
        assert g.read_state() == c.state
        _, peg = g.kicks()
        _, pec = c.kicks()
        assert abs(peg - pec) < 1e-4 * max(abs(pec), 1.0)


def test_bond_kicks_at_the_edges_match_the_oracle(O):
    """A harmonic bond, a zero-length tether, a FENE bond stretched past its 0.999999 cap (its
    kick saturates), a bond across the periodic boundary and one longer than 8 sigma (the
    separation's long form), with two masses: kicks and one step equal the oracle's."""
    tiny = Pair(1.0, 0.1, 0.1 * 2 ** (1 / 6))
    sys_ = System([int(40 * ONE), int(40 * ONE)], 0.005, tiny, [1.0, 2.0])
    types = [Bond.harmonic(50.0, 1.0), Bond.harmonic(3.0, 0.0), Bond.fene_bond(30.0, 1.5)]
    pos = np.array([[5, 5], [6.3, 5.4], [20, 20], [20.7, 21.1], [30, 30], [31.6, 30.05], [2, 2], [38.5, 39.2], [10, 30], [19.5, 31]])
    pos = (pos * ONE).astype(np.int64)
    bonds = [(0, 1, 0), (2, 3, 1), (4, 5, 2), (6, 7, 0), (8, 9, 1)]
    sys_.with_bonds(types, bonds)
    sp = np.array([0, 1, 0, 1, 0, 1, 1, 0, 0, 1], np.uint32)
    st = State(pos, np.zeros((10, 2), np.int32), sp)
    c = O.IntEngine(sys_, st)
    with GpuEngine(sys_, st, ForceMode.cell_list()) as g:
        kg, _ = g.kicks()
        kc, _ = c.kicks()
        assert np.array_equal(kg, kc)
        g.step(1)
        c.step(1)
        assert g.read_state() == c.state


def test_bonds_are_checked(O):
    """Bonds are 2D (GBMD_E_UNSUPPORTED in 3D); a bond needs two particles and a known type, and a
    particle at most four bonds (GBMD_E_INVALID)."""
    from micrographia_gb300 import _abi

    sys3 = System3(cube_for(500, 0.5), 0.005, Pair.wca(), [1.0])
    s3 = O.fcc_maxwell(sys3, 500, 1.0, 1)
    with GpuEngine3(sys3, s3, ForceMode.verlet_with_skin(sys3, 500, 0.3)) as g:
        with pytest.raises(RuntimeError) as err:
            g.set_bonds([Bond.kremer_grest()], [(0, 1, 0)])
        assert "two-dimensional" in str(err.value)
    sys_, s0 = _melt(O, 4, 10, 0.3, 1)
    with GpuEngine(sys_, s0, ForceMode.cell_list()) as g:
        for bad in ([(0, 0, 0)], [(0, 1, 1)], [(0, k, 0) for k in range(1, 6)], [(0, 40, 0)]):
            with pytest.raises(RuntimeError):
                g.set_bonds([Bond.kremer_grest()], bad)


@pytest.mark.parametrize("mode", ["cells", "verlet"])
def test_bonds_added_and_removed_between_steps(O, mode):
    """GpuEngine::add_bond / remove_bond (engine.rs:976-1012): a chain cut in the middle, two chain
    ends joined and two beads of a chain bonded, with a second (harmonic) bond type, between steps;
    the oracle's partner table is rebuilt from the same bond list, and the runs stay bit-identical
    (cells, and Verlet lists with the force kernel's epilogue)."""
    from micrographia_gb300 import Bond, _abi

    sys_, s0 = _melt(O, 20, 20, 0.3, 7)
    types = [Bond.kremer_grest(), Bond.harmonic(20.0, 1.2)]
    sys_.with_bonds(types, sys_.bonds)
    bonds = list(sys_.bonds)
    m = ForceMode.cell_list() if mode == "cells" else ForceMode.verlet_with_skin(sys_, s0.n(), 0.3)
    c = O.IntEngine(sys_, s0)
    with GpuEngine(sys_, s0, m, flags=_abi.force_lanes_flag(1)) as g:
        g.step(300)
        c.step(300)
        assert g.remove_bond(9, 10)
        assert not g.remove_bond(9, 10)
        assert g.add_bond(19, 20, 1)  # the end of chain 0 to the start of chain 1 (harmonic)
        assert g.add_bond(45, 47, 1)
        assert not g.add_bond(45, 47, 1)  # already bonded
        bonds = [b for b in bonds if {b[0], b[1]} != {9, 10}] + [(19, 20, 1), (45, 47, 1)]
        c.set_bonds([("fene" if t.fene else "harmonic", t.k, t.r0) for t in types], bonds)
        g.step(500)
        c.step(500)
        assert g.read_state() == c.state
        kg, _ = g.kicks()
        kc, _ = c.kicks()
        assert np.array_equal(kg, kc)
