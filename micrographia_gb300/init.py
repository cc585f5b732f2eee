"""Seeded initial conditions, generated on the device (gbmd_init_state, gbmd_maxwell): the mirror
of md-core's init.rs (fluid: lattice + maxwell, 1 sigma clear of any walls; maxwell for given
species) and three.rs (fcc + maxwell), plus this engine's triangular lattice and liquid-vapour
slab. Bit-identical to the CPU definitions."""

import ctypes as C
import math

import numpy as np

from . import _abi
from .core import DT, UNIT, Pair, State, System, System3, box_for, cube_for, to_f64, to_fixed  # noqa: F401
from .engine import init_state
from .workloads import uniform

STREAM_VELOCITY = 1
STREAM_JITTER = 2
STREAM_DIRECTION = 3


def fluid(sys: System, n, t, seed):
    """init::fluid (init.rs:107-121) on a periodic box: lattice with jitter 0.1 + Maxwell at t."""
    return init_state(sys, _abi.INIT_FLUID, n, t, seed, jitter=0.1)


def maxwell(sys, species, t, seed):
    """init::maxwell (init.rs:42-57) / three::maxwell: velocities for these id-ordered species,
    each at kT = t with its own mass, with the exact zero velocity sum (on the device)."""
    sp = np.ascontiguousarray(species, dtype=np.uint32)
    vel = np.empty((sp.size, sys.DIM), np.int32)
    csys = sys.to_c()
    _abi.check(
        _abi.lib().gbmd_maxwell(C.byref(csys), sp.ctypes.data_as(C.POINTER(C.c_uint32)), sp.size, float(t), int(seed),
                                vel.ctypes.data_as(C.POINTER(C.c_int32)))
    )
    return vel


def fixed_speed(sys, species, t, seed):
    """init::fixed_speed (init.rs:61-74), 2D: every particle at speed sqrt(2 t / m) in a random
    direction (fdlibm cos and sin, on the device), with the exact zero velocity sum."""
    sp = np.ascontiguousarray(species, dtype=np.uint32)
    vel = np.empty((sp.size, 2), np.int32)
    csys = sys.to_c()
    _abi.check(
        _abi.lib().gbmd_fixed_speed(C.byref(csys), sp.ctypes.data_as(C.POINTER(C.c_uint32)), sp.size, float(t), int(seed),
                                    vel.ctypes.data_as(C.POINTER(C.c_int32)))
    )
    return vel


def lattice(n, box_len, jitter, seed):
    """init::lattice (init.rs:22-38): the first n sites of a square-ish lattice filling the 2D box,
    jittered (on the device)."""
    sys_ = System([int(box_len[0]), int(box_len[1])], DT, Pair.wca(), [1.0])
    return init_state(sys_, _abi.INIT_FLUID, n, 1.0, seed, jitter=jitter).pos


def _moving(sys, species):
    sp = np.asarray(species, dtype=np.uint32)
    if sys is None or sys.DIM == 2:
        return np.arange(sp.size)
    return np.nonzero(((sys.pinned >> sp.astype(np.int64)) & 1) == 0)[0]


def zero_velocity_sum(vel, sys=None, species=None):
    """init::zero_velocity_sum (init.rs:76-89) and three::zero_velocity_sum (three.rs:376-390), in
    place: per axis the integer sum S over the particles (3D: the moving ones), q = S div n and
    r = S mod n (Euclidean), and particle k of them loses q + (k < r)."""
    idx = _moving(sys, species if species is not None else np.zeros(len(vel), np.uint32))
    n = idx.size
    if n == 0:
        return vel
    for a in range(vel.shape[1]):
        total = int(vel[idx, a].astype(np.int64).sum())
        q, r = divmod(total, n)
        sub = q + (np.arange(n) < r).astype(np.int64)
        vel[idx, a] = (vel[idx, a].astype(np.int64) - sub).astype(np.int32)
    return vel


def half_step_kinetic(sys, state):
    """State::half_step_kinetic (system.rs:505-515) / State3's (three.rs:299-308, moving particles
    only): sum of 1/2 m |v|^2, v = v_int UNIT / dt, added in id order in f64."""
    v = state.vel.astype(np.float64) * UNIT / sys.dt
    sq = v * v
    acc = sq[:, 0] + sq[:, 1]
    if sys.DIM == 3:
        acc = acc + sq[:, 2]
    m = np.asarray(sys.masses, np.float64)[state.species]
    terms = 0.5 * m * acc
    if sys.DIM == 3:
        terms = terms[_moving(sys, state.species)]
    return float(np.add.accumulate(terms)[-1]) if terms.size else 0.0


def _round_i32(x):
    """f64::round (half away from zero) then `as i32` (saturating, NaN to 0)."""
    r = np.trunc(x)
    r = r + np.where(np.abs(x - r) >= 0.5, np.sign(x), 0.0)
    r = np.where(np.isnan(r), 0.0, r)
    return np.clip(r, -2147483648.0, 2147483647.0).astype(np.int32)


def set_temperature(state, sys, t):
    """init::set_temperature (init.rs:92-103) / three::set_temperature (three.rs:392-404), in
    place: velocities scaled by sqrt(t / T_now), T_now the half-step kinetic temperature (dof
    n - 1 in 2D, 1.5 (moving - 1) in 3D), rounded, then the exact zero sum."""
    if sys.DIM == 2:
        dof = max(state.n() - 1.0, 1.0)
    else:
        dof = 1.5 * max(_moving(sys, state.species).size - 1.0, 1.0)
    now = half_step_kinetic(sys, state) / dof
    if now <= 0.0:
        return state
    f = math.sqrt(t / now)
    state.vel = _round_i32(state.vel.astype(np.float64) * f)
    zero_velocity_sum(state.vel, sys, state.species)
    return state


def compartment_fluid(sys, per_box, t, seed):
    """init::compartment_fluid (init.rs:126-149): per_box particles on a small jittered lattice in
    every compartment, 0.6 sigma clear of its walls, numbered box by box (row-major), with Maxwell
    velocities at t."""
    cx, cy = sys.compartment_counts()
    side = [to_f64(sys.box_len[0]) / cx, to_f64(sys.box_len[1]) / cy]
    nx = max(int(math.ceil(math.sqrt(per_box * side[0] / side[1]))), 1)
    ny = -(-per_box // nx)
    margin = 0.6
    a = [(side[0] - 2.0 * margin) / nx, (side[1] - 2.0 * margin) / ny]
    pos = []
    for by in range(cy):
        for bx in range(cx):
            for k in range(per_box):
                i = len(pos)
                jx = 0.2 * a[0] * (uniform(seed, STREAM_JITTER, 2 * i) - 0.5)
                jy = 0.2 * a[1] * (uniform(seed, STREAM_JITTER, 2 * i + 1) - 0.5)
                x = bx * side[0] + margin + ((k % nx) + 0.5) * a[0] + jx
                y = by * side[1] + margin + ((k // nx) + 0.5) * a[1] + jy
                pos.append([to_fixed(x), to_fixed(y)])
    sp = np.zeros(len(pos), np.uint32)
    return State(np.array(pos, np.int64).reshape(-1, 2), maxwell(sys, sp, t, seed), sp)


def mark_disc(state, sys, center, radius, species):
    """init::mark_disc (init.rs:152-163), in place: the particles within `radius` sigma of
    `center` (sigma, minimum image) take `species`."""
    c = [to_fixed(center[0]), to_fixed(center[1])]
    d2 = np.zeros(state.n())
    for a in range(2):
        f = _min_image(c[a], state.pos[:, a], sys.box_len[a]).astype(np.float64) * UNIT
        d2 = d2 + f * f if a else f * f
    state.species[d2 < radius * radius] = species
    return state


def _min_image(a, b, L):
    """fixed::min_image (fixed.rs:31-40): d = b - a, less L at or above L/2, plus L below -L/2."""
    d = np.asarray(b, np.int64) - np.int64(a)
    half = L // 2
    return np.where(d >= half, d - L, np.where(d < -half, d + L, d))


def barometric(sys, species, t, min_sep, margin, seed):
    """init::barometric (init.rs:223-260): heights drawn from exp(-m g y / kT) between `margin`
    and the box top less `margin`, x uniform, rejecting draws closer than `min_sep` sigma to a
    placed particle (x periodic), draws numbered across all attempts; Maxwell velocities at t."""
    sp = np.ascontiguousarray(species, np.uint32)
    return State(barometric_positions(sys, sp, t, min_sep, margin, seed), maxwell(sys, sp, t, seed), sp.copy())


def barometric_positions(sys, species, t, min_sep, margin, seed):
    """The positions of `barometric` (host only; the draws and the rejection in f64, exp and ln
    from the platform's libm as the reference's f64::exp and f64::ln)."""
    b = [to_f64(sys.box_len[0]), to_f64(sys.box_len[1])]
    g = -sys.gravity[1]
    h = b[1] - 2.0 * margin
    cell = max(min_sep, 0.5)
    gx, gy = int(math.ceil(b[0] / cell)), int(math.ceil(b[1] / cell))
    grid = [[] for _ in range(gx * gy)]
    pos = []
    draw = 0
    sp = np.asarray(species, np.uint32)
    for s in sp:
        lam = sys.masses[int(s)] * g / t
        while True:
            ux = uniform(seed, STREAM_JITTER, draw)
            uy = uniform(seed, STREAM_DIRECTION, draw)
            draw += 1
            x = ux * b[0]
            y = margin + (-math.log(1.0 - uy * (1.0 - math.exp(-lam * h))) / lam if lam > 1e-12 else uy * h)
            cx, cy = min(int(x / cell), gx - 1), min(int(y / cell), gy - 1)
            clash = False
            for yy in range(max(cy - 1, 0), min(cy + 2, gy)):
                for ox in range(3):
                    xx = (cx + gx + ox - 1) % gx
                    for j in grid[yy * gx + xx]:
                        dx = abs(pos[j][0] - x)
                        dx = min(dx, b[0] - dx)
                        dy = pos[j][1] - y
                        if dx * dx + dy * dy < min_sep * min_sep:
                            clash = True
                            break
                    if clash:
                        break
                if clash:
                    break
            if not clash:
                grid[cy * gx + cx].append(len(pos))
                pos.append([x, y])
                break
    return np.array([[to_fixed(q[0]), to_fixed(q[1])] for q in pos], np.int64).reshape(-1, 2)


def triangular(sys: System, n, t, seed, jitter=0.1):
    """Triangular lattice + Maxwell (2D)."""
    return init_state(sys, _abi.INIT_TRIANGULAR, n, t, seed, jitter=jitter)


def fcc_maxwell(sys: System3, n, t, seed, jitter=0.05):
    """three::fcc on fcc_cells(n, box) + three::maxwell at t with the same seed."""
    return init_state(sys, _abi.INIT_FCC, n, t, seed, jitter=jitter)


def slab(sys: System, n, t, seed, rho_liquid=0.7, rho_vapour=0.05, frac=0.25, jitter=0.1):
    """Liquid slab (triangular, rho_liquid) across x in [L(1-f)/2, L(1+f)/2) and a jittered
    lattice of vapour at rho_vapour elsewhere; Maxwell at t."""
    return init_state(sys, _abi.INIT_SLAB, n, t, seed, jitter=jitter, rho_liquid=rho_liquid, rho_vapour=rho_vapour, slab_frac=frac)
