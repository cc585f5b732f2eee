"""The Observer's reading and the two measures computed from it (crates/md/src/observe.rs).

`GpuEngine.observe_grid(grid, marked)` returns a `Reading`: particle counts on a gx x gy grid
over the box (row-major, bin by * gx + bx), the same counts for the marked species, and the
half-step kinetic energy. `mixing` and `segregation` reduce a reading to one number each, in
f64 in the reference's order of operations.
"""

import math
from dataclasses import dataclass

import numpy as np


def _div(a, b):
    """a / b with IEEE semantics (as Rust's f64 division): +-inf for b = 0, NaN for 0 / 0."""
    if b != 0.0:
        return a / b
    if a == 0.0 or math.isnan(a):
        return math.nan
    return math.copysign(math.inf, a) * math.copysign(1.0, b)


def _clamp01(x):
    """f64::clamp(0.0, 1.0): NaN stays NaN."""
    return x if math.isnan(x) else min(max(x, 0.0), 1.0)


@dataclass
class Reading:
    """observe.rs:38-44: counts of all particles and of the marked species per bin, and the
    kinetic energy."""

    all: np.ndarray
    marked: np.ndarray
    kinetic: float


def mixing(r):
    """observe.rs:134-155: 1 - D / D_max, clamped to [0, 1], where D = sum p ln(p / q) is the
    relative entropy of the marked particles' distribution p over the bins with respect to all
    particles' q, and D_max = ln(all / marked). 0 when there is nothing to measure; NaN when every
    particle is marked (0 / 0, as in the reference's f64 arithmetic)."""
    total = sum(float(c) for c in r.marked)
    alln = sum(float(c) for c in r.all)
    if total == 0.0 or alln == 0.0:
        return 0.0
    d = 0.0
    for m, a in zip(r.marked, r.all):
        if m > 0:
            p = float(m) / total
            q = float(a) / alln
            d += p * math.log(p / q)
    d_max = math.log(alln / total)
    return _clamp01(1.0 - _div(d, d_max))


def segregation(r):
    """observe.rs:157-181: the particle-weighted variance of the bins' marked fraction in excess
    of binomial noise, over its maximum f (1 - f), clamped to [0, 1]; 0 when either kind is
    absent; NaN when no bin holds two particles (the noise then equals the maximum: 0 / 0)."""
    n = m = 0.0
    for a, k in zip(r.all, r.marked):
        n += float(a)
        m += float(k)
    if n == 0.0 or m == 0.0 or m == n:
        return 0.0
    f = m / n
    var = noise = 0.0
    for a, k in zip(r.all, r.marked):
        a = float(a)
        if a > 0.0:
            fb = float(k) / a
            var += a * (fb - f) ** 2
            noise += f * (1.0 - f)
    var /= n
    noise /= n
    mx = f * (1.0 - f)
    return _clamp01(_div(var - noise, mx - noise))
