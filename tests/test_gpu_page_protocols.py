"""The reference's page-parameter protocols on the GPU engine (crates/md/tests/gpu_engine.rs:
185-253): chaos from a one-bit flip, the nudged reversal, and storage reordering."""

import math

import numpy as np
import pytest

from micrographia_gb300 import DT, ForceMode, GpuEngine, Pair, System, box_for, init

pytestmark = pytest.mark.gpu


def _page_state():
    """gpu_engine.rs:188-194: 8000 WCA discs at density 0.5 in a 4:3 box, 1000 warm-up steps,
    rescaled to T = 1 (init::set_temperature)."""
    n = 8000
    sys_ = System(box_for(n, 0.5, 4.0 / 3.0), DT, Pair.wca(), [1.0])
    s0 = init.fluid(sys_, n, 1.0, 7)
    with GpuEngine(sys_, s0) as warm:
        warm.step(1000)
        s0 = warm.read_state()
    init.set_temperature(s0, sys_, 1.0)
    return sys_, s0


def test_one_bit_flip_grows_exponentially():
    """gpu_engine.rs:185-216: two runs a single low bit apart; the largest deviation grows
    exponentially (the fitted rate of ln max over the window 0 < max < 0.05 sigma is positive and
    of order one per tau) until the runs decorrelate."""
    sys_, s0 = _page_state()
    fit = []
    with GpuEngine(sys_, s0) as a, GpuEngine(sys_, s0) as b:
        b.flip_bit(0, 0, 0)
        last = 0
        for k in range(1, 41):
            a.step(100)
            b.step(100)
            differ, mx = a.read_state().position_difference(b.read_state(), sys_)
            t = k * 100.0 * DT
            if 0.0 < mx < 0.05:
                fit.append((t, math.log(mx)))
            last = differ
    assert len(fit) >= 4
    mt = sum(f[0] for f in fit) / len(fit)
    my = sum(f[1] for f in fit) / len(fit)
    slope = sum((f[0] - mt) * (f[1] - my) for f in fit) / sum((f[0] - mt) ** 2 for f in fit)
    assert 0.3 < slope < 20.0, slope
    assert last > 1000  # the deviation has spread through the fluid


def test_nudged_reversal_misses_by_more_the_longer_the_run():
    """gpu_engine.rs:218-240: forward, flip one bit, reverse, back to t = 0. The unflipped run
    returns exactly; the nudged one misses the start, by more after a longer forward run."""
    sys_, s0 = _page_state()
    miss = []
    for steps in (1000, 3000, 6000):
        with GpuEngine(sys_, s0) as e:
            e.step(steps)
            e.flip_bit(0, 0, 0)
            e.reverse()
            e.step(steps)
            e.reverse()
            differ, mx = e.read_state().position_difference(s0, sys_)
        miss.append((differ, mx))
    with GpuEngine(sys_, s0) as e:
        e.step(3000)
        e.reverse()
        e.step(3000)
        e.reverse()
        assert e.read_state() == s0
    assert all(d > 0 for d, _ in miss)
    assert miss[0][1] < miss[2][1]


def test_storage_reordering_does_not_change_the_trajectory():
    """gpu_engine.rs:242-253 with this engine's reordering: a cell-list run re-sorted into cell
    order every 7 steps (sort_now) and one never re-sorted between steps end with the same hash."""
    n = 6000
    sys_ = System(box_for(n, 0.6, 1.0), DT, Pair.lj(2.5), [1.0])
    s0 = init.fluid(sys_, n, 1.0, 9)
    with GpuEngine(sys_, s0, ForceMode.cell_list()) as a, GpuEngine(sys_, s0, ForceMode.cell_list()) as b:
        a.step(1500)
        done = 0
        while done < 1500:
            k = min(7, 1500 - done)
            b.step(k)
            b.sort_now()
            done += k
        assert a.read_state().hash() == b.read_state().hash()
