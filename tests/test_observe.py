"""The Observer (crates/md/src/observe.rs): mixing and segregation on hand-made readings, and the
oracle's density grid against a numpy float32 restatement of observe.wgsl:25-45 (no GPU)."""

import math

import numpy as np
import pytest

from micrographia_gb300 import ONE, Pair, Reading, State, System, mixing, segregation


def _r(all_, marked):
    return Reading(np.array(all_, np.uint32), np.array(marked, np.uint32), 0.0)


def test_mixing_and_segregation_at_their_ends():
    """Marked in proportion to all: mixing 1, segregation 0. Marked alone in half the bins:
    mixing 0, segregation 1. Nothing marked, or nothing at all: 0 for both (observe.rs:136-139,
    162-164)."""
    mixed = _r([40, 20, 60, 80], [10, 5, 15, 20])
    assert mixing(mixed) == 1.0
    assert segregation(mixed) == 0.0
    apart = _r([10, 10], [10, 0])
    assert mixing(apart) == 0.0
    assert segregation(apart) == 1.0
    for r in (_r([3, 4], [0, 0]), _r([0, 0], [0, 0]), _r([5, 5], [5, 5])):
        assert segregation(r) == 0.0
    assert mixing(_r([3, 4], [0, 0])) == 0.0


def test_mixing_and_segregation_zero_over_zero():
    """Where the reference divides 0 by 0 the result is NaN, as Rust's f64 gives (clamp keeps
    NaN): segregation when no bin holds two particles, mixing when every particle is marked."""
    assert math.isnan(segregation(_r([1, 1, 0, 1], [1, 0, 0, 0])))
    assert math.isnan(mixing(_r([4, 6], [4, 6])))


def test_mixing_and_segregation_in_between():
    """A partial case against the formulas written out: D = sum p ln(p/q), 1 - D/ln(N/M); the
    excess variance over binomial noise, over f(1 - f) minus the noise."""
    all_, mk = [30, 50, 20, 0], [20, 10, 0, 0]
    n, m = 100.0, 30.0
    d = sum((k / m) * math.log((k / m) / (a / n)) for a, k in zip(all_, mk) if k)
    assert abs(mixing(_r(all_, mk)) - (1.0 - d / math.log(n / m))) < 1e-15
    f = m / n
    var = sum(a * (k / a - f) ** 2 for a, k in zip(all_, mk) if a) / n
    noise = 3 * f * (1 - f) / n
    want = (var - noise) / (f * (1 - f) - noise)
    assert abs(segregation(_r(all_, mk)) - want) < 1e-15


def _grid_f32(sys_, st, gx, gy, marked):
    """observe.wgsl:25-45 in numpy float32: coord = f32(hi) + f32(lo) 2^-32, times (g / L) as f32,
    truncated and clamped to g - 1."""
    out = []
    for a, g in ((0, gx), (1, gy)):
        x = st.pos[:, a].astype(np.int64) % sys_.box_len[a]
        u = x.astype(np.uint64)
        hi = (u >> np.uint64(32)).astype(np.uint32).astype(np.float32)
        lo = (u & np.uint64(0xFFFFFFFF)).astype(np.uint32).astype(np.float32) * np.float32(2.0**-32)
        c = hi + lo
        s = np.float32(g / (sys_.box_len[a] / ONE))
        out.append(np.minimum((c * s).astype(np.uint32), g - 1))
    b = out[1].astype(np.int64) * gx + out[0]
    all_ = np.bincount(b, minlength=gx * gy).astype(np.uint32)
    mk = np.bincount(b[st.species == marked], minlength=gx * gy).astype(np.uint32)
    return all_, mk


@pytest.mark.parametrize("grid", [(1, 1), (16, 12), (7, 200)])
def test_oracle_grid_matches_the_shader_restatement(O, grid):
    """Random positions, including the last representable positions below L (where the f32
    coordinate rounds up to L and the clamp takes the bin) and exact bin edges."""
    rng = np.random.default_rng(5)
    sys_ = System([int(37.5 * ONE), int(21.25 * ONE)], 0.005, Pair.wca(), [1.0, 1.0])
    n = 5000
    pos = np.stack([rng.integers(0, sys_.box_len[0], n), rng.integers(0, sys_.box_len[1], n)], axis=1).astype(np.int64)
    pos[:8, 0] = sys_.box_len[0] - np.arange(1, 9)
    pos[8:16, 1] = sys_.box_len[1] - np.arange(1, 9)
    edges = (np.arange(16) % grid[0]) * sys_.box_len[0] // grid[0]
    pos[16:32, 0] = edges
    sp = (rng.random(n) < 0.3).astype(np.uint32)
    st = State(pos, np.zeros((n, 2), np.int32), sp)
    ga, gm = O.observer_grid(sys_, st, grid, 1)
    wa, wm = _grid_f32(sys_, st, grid[0], grid[1], 1)
    assert np.array_equal(ga, wa)
    assert np.array_equal(gm, wm)
    assert ga.sum() == n and gm.sum() == sp.sum()
