"""ORACLE — test infrastructure only (the CPU restatement of micrographia's md-ref / md-core).

ctypes bindings of oracle/_build/liboracle.so for the parity tests, __graft_entry__.smoke() and
bench.py's CPU baseline. The engine package never imports this module.
"""

import ctypes as C
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from micrographia_gb300 import _abi  # noqa: E402  (ABI struct definitions only)
from micrographia_gb300.core import State, State3  # noqa: E402

from . import build as _build  # noqa: E402

P = C.POINTER
VP = C.c_void_p
I64P, I32P, U32P, U64P, DP = P(C.c_int64), P(C.c_int32), P(C.c_uint32), P(C.c_uint64), P(C.c_double)
SYS = P(_abi.gbmd_system)

_SIGS = [
    ("oracle_sep_f32", C.c_int, [C.c_int64, P(C.c_float)]),
    ("oracle_sep_near", C.c_float, [C.c_int64]),
    ("oracle_threefry", None, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, U32P]),
    ("oracle_uniform", C.c_double, [C.c_uint64, C.c_uint32, C.c_uint32]),
    ("oracle_normal", C.c_double, [C.c_uint64, C.c_uint32, C.c_uint32]),
    ("oracle_log", C.c_double, [C.c_double]),
    ("oracle_cos", C.c_double, [C.c_double]),
    ("oracle_sin", C.c_double, [C.c_double]),
    ("oracle_libm_compare", None, [C.c_uint64, C.c_uint64, C.c_double, C.c_double, U64P]),
    ("oracle_fdlibm_many", None, [DP, C.c_uint64, DP]),
    ("oracle_to_fixed", C.c_int64, [C.c_double]),
    ("oracle_box_for", None, [C.c_uint64, C.c_double, C.c_double, I64P]),
    ("oracle_cube_for", None, [C.c_uint64, C.c_double, I64P]),
    ("oracle_fcc_cells", None, [C.c_uint64, I64P, U64P]),
    ("oracle_cells_for", C.c_int, [SYS, C.c_double, U32P]),
    ("oracle_wca_rc", C.c_double, []),
    ("oracle_pair_shift", C.c_double, [C.c_double, C.c_double, C.c_double]),
    ("oracle_lattice", None, [C.c_uint64, I64P, C.c_double, C.c_uint64, I64P]),
    ("oracle_fcc", None, [C.c_uint64, I64P, U64P, C.c_double, C.c_uint64, I64P]),
    ("oracle_maxwell", None, [SYS, U32P, C.c_uint64, C.c_double, C.c_uint64, I32P]),
    ("oracle_zero_velocity_sum", None, [SYS, U32P, C.c_uint64, I32P]),
    ("oracle_set_temperature", None, [SYS, I32P, U32P, C.c_uint64, C.c_double, C.c_int]),
    ("oracle_exact_kinetic", C.c_double, [SYS, I32P, U32P, C.c_uint64]),
    ("oracle_half_step_kinetic", C.c_double, [SYS, I32P, U32P, C.c_uint64]),
    ("oracle_init", C.c_int, [SYS, P(_abi.gbmd_init), I64P, I32P, U32P]),
    ("oracle_cell_list", C.c_int, [SYS, I64P, C.c_uint64, U32P, U32P, U32P, U32P]),
    ("oracle_verlet_cap", C.c_uint32, [SYS, C.c_uint64, C.c_double]),
    ("oracle_verlet_list", C.c_int64, [SYS, I64P, U32P, C.c_uint64, C.c_double, U32P, U32P, C.c_uint64]),
    ("oracle_verlet_list_of", C.c_int64, [SYS, I64P, U32P, C.c_uint64, C.c_double, U32P, C.c_uint64, C.c_int, U32P, U32P, C.c_uint64]),
    ("oracle_engine_create", VP, [SYS, I64P, I32P, U32P, C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int]),
    ("oracle_engine_destroy", None, [VP]),
    ("oracle_engine_set_half3", None, [VP, C.c_int]),
    ("oracle_engine_step", None, [VP, C.c_uint64]),
    ("oracle_engine_reverse", None, [VP]),
    ("oracle_engine_kicks", C.c_double, [VP, I32P]),
    ("oracle_engine_kicks_of", None, [VP, U32P, C.c_uint64, I32P]),
    ("oracle_engine_state", None, [VP, I64P, I32P, U32P]),
    ("oracle_engine_set_state", None, [VP, I64P, I32P, U32P]),
    ("oracle_engine_hash", C.c_uint64, [VP]),
    ("oracle_engine_ledger", None, [VP, DP, I64P, U64P, U32P]),
    ("oracle_engine_set_system", None, [VP, SYS]),
    ("oracle_engine_wall_ledger", None, [VP, DP, DP, U64P]),
    ("oracle_engine_wall_ledger_fixed", None, [VP, I64P, I64P]),
    ("oracle_engine_set_bonds", None, [VP, U32P, DP, DP, C.c_uint32, U32P, C.c_uint64]),
    ("oracle_engine_set_piston", C.c_int, [VP, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]),
    ("oracle_engine_piston", None, [VP, I64P, I32P, DP, DP]),
    ("oracle_engine_set_piston_speed", None, [VP, C.c_double]),
    ("oracle_engine_compartment_ledger", C.c_uint32, [VP, I64P, I64P, U64P]),
    ("oracle_engine_steps", C.c_int64, [VP]),
    ("oracle_engine_energy", None, [VP, DP, DP]),
    ("oracle_state_hash", C.c_uint64, [C.c_uint32, I64P, I32P, U32P, C.c_uint64]),
    ("oracle_float_create", VP, [SYS, I64P, I32P, U32P, C.c_uint64]),
    ("oracle_float_destroy", None, [VP]),
    ("oracle_float_step", None, [VP, C.c_uint64]),
    ("oracle_float_positions", None, [VP, DP]),
    ("oracle_float_energy", None, [VP, DP, DP]),
    ("oracle_pair_sums", None, [SYS, I64P, U32P, C.c_uint64, DP, DP]),
    ("oracle_rdf", None, [SYS, I64P, C.c_uint64, C.c_uint32, C.c_double, U64P]),
    ("oracle_profile", None, [SYS, I64P, C.c_uint64, C.c_uint32, C.c_uint32, U64P]),
    ("oracle_fixed_speed", None, [SYS, U32P, C.c_uint64, C.c_double, C.c_uint64, I32P]),
    ("oracle_barometric", None, [SYS, U32P, C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_uint64, I64P]),
    ("oracle_mark_disc", None, [SYS, I64P, U32P, C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_uint32]),
    ("oracle_observer_grid", None, [SYS, I64P, U32P, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, U32P]),
    ("oracle_int_kick", C.c_int, [SYS, C.c_uint32, C.c_uint32, I64P, I32P]),
]

_lib = None


def lib():
    global _lib
    if _lib is None:
        l = C.CDLL(_build.build())
        for name, res, args in _SIGS:
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def _p(a, t):
    return a.ctypes.data_as(P(t))


def threefry(ctr, key, rounds=20):
    out = (C.c_uint32 * 2)()
    lib().oracle_threefry(ctr[0], ctr[1], key[0], key[1], rounds, out)
    return [out[0], out[1]]


def sep_f32(d):
    f = C.c_float()
    ok = lib().oracle_sep_f32(d, C.byref(f))
    return f.value if ok else None


def box_for(n, density, aspect=1.0):
    out = (C.c_int64 * 2)()
    lib().oracle_box_for(n, density, aspect, out)
    return [out[0], out[1]]


def cube_for(n, density):
    out = (C.c_int64 * 3)()
    lib().oracle_cube_for(n, density, out)
    return [out[0], out[1], out[2]]


def fcc_cells(n, box):
    b = (C.c_int64 * 3)(*box)
    out = (C.c_uint64 * 3)()
    lib().oracle_fcc_cells(n, b, out)
    return [out[0], out[1], out[2]]


def init(sys, spec):
    """The recipes of gbmd_init_state restated on the CPU."""
    n, D = spec.n, sys.DIM
    pos = np.empty((n, D), np.int64)
    vel = np.empty((n, D), np.int32)
    sp = np.empty(n, np.uint32)
    c = sys.to_c()
    if lib().oracle_init(C.byref(c), C.byref(spec), _p(pos, C.c_int64), _p(vel, C.c_int32), _p(sp, C.c_uint32)) != 0:
        raise ValueError("oracle init failed")
    return (State if D == 2 else State3)(pos, vel, sp)


def fdlibm_many(x):
    """fdlibm's (ln, cos, sin) at each of x: an (n, 3) array."""
    x = np.ascontiguousarray(x, np.float64)
    out = np.empty((x.size, 3), np.float64)
    lib().oracle_fdlibm_many(_p(x, C.c_double), x.size, _p(out, C.c_double))
    return out


def libm_compare(n, seed, t_over_m, dt):
    """oracle_libm_compare: over n of the heat bath's 2D draws, how often fdlibm's ln, cos and sin
    and the platform libm's round differently, and how many draws' step displacements differ."""
    out = (C.c_uint64 * 4)()
    lib().oracle_libm_compare(n, seed, t_over_m, dt, out)
    return list(out)


def fluid(sys, n, t, seed):
    """init::fluid (periodic)."""
    from micrographia_gb300.engine import make_init

    return init(sys, make_init(_abi.INIT_FLUID, n, t, seed, jitter=0.1))


def fcc_maxwell(sys, n, t, seed, jitter=0.05):
    from micrographia_gb300.engine import make_init

    return init(sys, make_init(_abi.INIT_FCC, n, t, seed, jitter=jitter))


def maxwell(sys, species, t, seed):
    species = np.ascontiguousarray(species, np.uint32)
    vel = np.empty((len(species), sys.DIM), np.int32)
    c = sys.to_c()
    lib().oracle_maxwell(C.byref(c), _p(species, C.c_uint32), len(species), t, seed, _p(vel, C.c_int32))
    return vel


def set_temperature(sys, state, t, exact=False):
    vel = np.ascontiguousarray(state.vel.copy())
    c = sys.to_c()
    lib().oracle_set_temperature(C.byref(c), _p(vel, C.c_int32), _p(state.species, C.c_uint32), state.n(), t, 1 if exact else 0)
    return vel


def cell_list(sys, state, dims):
    n = state.n()
    d = list(dims) + [1] * (3 - len(dims))
    ncell = int(np.prod(d[: sys.DIM]))
    keys = np.empty(n, np.uint32)
    start = np.empty(ncell + 1, np.uint32)
    items = np.empty(n, np.uint32)
    c = sys.to_c()
    dd = (C.c_uint32 * 3)(*d)
    lib().oracle_cell_list(C.byref(c), _p(state.pos, C.c_int64), n, dd, _p(keys, C.c_uint32), _p(start, C.c_uint32), _p(items, C.c_uint32))
    return keys, start, items


def verlet_lists(sys, state, skin):
    n = state.n()
    counts = np.empty(n, np.uint32)
    cap = n * 512
    nbr = np.empty(cap, np.uint32)
    c = sys.to_c()
    tot = lib().oracle_verlet_list(C.byref(c), _p(state.pos, C.c_int64), _p(state.species, C.c_uint32), n, skin, _p(counts, C.c_uint32), _p(nbr, C.c_uint32), cap)
    if tot < 0:
        raise ValueError("list buffer too small")
    offs = np.concatenate([[0], np.cumsum(counts.astype(np.int64))])
    return [nbr[offs[i] : offs[i + 1]].copy() for i in range(n)]


def verlet_lists_of(sys, state, skin, idx, threads=1):
    """The lists of the particles idx only (sorted neighbour indices each): a sample of a system
    too large to list whole within a test."""
    idx = np.ascontiguousarray(idx, np.uint32)
    m = len(idx)
    counts = np.empty(m, np.uint32)
    cap = m * 512
    nbr = np.empty(cap, np.uint32)
    c = sys.to_c()
    tot = lib().oracle_verlet_list_of(C.byref(c), _p(state.pos, C.c_int64), _p(state.species, C.c_uint32), state.n(), skin,
                                      _p(idx, C.c_uint32), m, threads, _p(counts, C.c_uint32), _p(nbr, C.c_uint32), cap)
    if tot < 0:
        raise ValueError("list buffer too small")
    offs = np.concatenate([[0], np.cumsum(counts.astype(np.int64))])
    return [nbr[offs[q] : offs[q + 1]].copy() for q in range(m)]


def pair_sums(sys, state):
    pe, w = C.c_double(), C.c_double()
    c = sys.to_c()
    lib().oracle_pair_sums(C.byref(c), _p(state.pos, C.c_int64), _p(state.species, C.c_uint32), state.n(), C.byref(pe), C.byref(w))
    return pe.value, w.value


def rdf(sys, state, bins, rmax):
    out = np.zeros(bins, np.uint64)
    c = sys.to_c()
    lib().oracle_rdf(C.byref(c), _p(state.pos, C.c_int64), state.n(), bins, rmax, _p(out, C.c_uint64))
    return out


def profile(sys, state, bins, axis):
    out = np.zeros(bins, np.uint64)
    c = sys.to_c()
    lib().oracle_profile(C.byref(c), _p(state.pos, C.c_int64), state.n(), bins, axis, _p(out, C.c_uint64))
    return out


def fixed_speed(sys, species, t, seed):
    """init::fixed_speed (init.rs:61-74)."""
    species = np.ascontiguousarray(species, np.uint32)
    vel = np.empty((len(species), 2), np.int32)
    c = sys.to_c()
    lib().oracle_fixed_speed(C.byref(c), _p(species, C.c_uint32), len(species), t, seed, _p(vel, C.c_int32))
    return vel


def barometric_positions(sys, species, t, min_sep, margin, seed):
    """init::barometric's positions (init.rs:223-260)."""
    species = np.ascontiguousarray(species, np.uint32)
    pos = np.empty((len(species), 2), np.int64)
    c = sys.to_c()
    lib().oracle_barometric(C.byref(c), _p(species, C.c_uint32), len(species), t, min_sep, margin, seed, _p(pos, C.c_int64))
    return pos


def mark_disc(sys, state, center, radius, species):
    """init::mark_disc (init.rs:152-163): the marked species array."""
    sp = state.species.copy()
    c = sys.to_c()
    lib().oracle_mark_disc(C.byref(c), _p(state.pos, C.c_int64), _p(sp, C.c_uint32), state.n(), center[0], center[1], radius, species)
    return sp


def observer_grid(sys, state, grid, marked):
    """Observer's counts (observe.wgsl:31-45): (all, marked), gx * gy each, row-major."""
    gx, gy = grid
    out = np.zeros(2 * gx * gy, np.uint32)
    c = sys.to_c()
    lib().oracle_observer_grid(C.byref(c), _p(state.pos, C.c_int64), _p(state.species, C.c_uint32), state.n(), gx, gy, marked, _p(out, C.c_uint32))
    return out[: gx * gy], out[gx * gy :]


def half_step_kinetic(sys, state):
    c = sys.to_c()
    return lib().oracle_half_step_kinetic(C.byref(c), _p(state.vel, C.c_int32), _p(state.species, C.c_uint32), state.n())


def exact_kinetic(sys, state):
    c = sys.to_c()
    return lib().oracle_exact_kinetic(C.byref(c), _p(state.vel, C.c_int32), _p(state.species, C.c_uint32), state.n())


# ---------------------------------------------------------------- page commands
def to_step_displacement(sys, v):
    """System::to_step_displacement (md-core system.rs:427-429): (v dt 2^32).round() as i32,
    Rust's round (half away from zero, exact) and saturating cast (NaN -> 0)."""
    x = float(v) * sys.dt * 4294967296.0
    if x != x:
        return 0
    r = math.trunc(x)
    if abs(x - r) >= 0.5:
        r += 1 if x > 0 else -1
    return int(min(max(r, -(1 << 31)), (1 << 31) - 1))


def _coord_f32(x):
    """coord_f32 (md/shaders/params.wgsl:117-119) of positions in [0, L): f32(hi) + ldexp(f32(lo), -32)."""
    u = x.astype(np.int64).view(np.uint64)
    hi = (u >> np.uint64(32)).astype(np.uint32).astype(np.float32)
    lo = (u & np.uint64(0xFFFFFFFF)).astype(np.uint32).astype(np.float32)
    return (hi + np.ldexp(lo, -32).astype(np.float32)).astype(np.float32)


def kick_region(sys, state, lo, hi, scale, add):
    """GpuEngine::kick_region (md/src/engine.rs:1026-1036) as md.wgsl:216-229 / md3.wgsl:541-553
    compute it: unpinned particles with lo <= coord_f32(x) < hi on every axis (f32 bounds) get
    v <- i32(round(f32(v) * f32(scale))) + add, round half to even, the sum wrapping."""
    d = sys.DIM
    out = state.copy()
    sel = ((sys.pinned >> state.species.astype(np.int64)) & 1) == 0
    for a in range(d):
        c = _coord_f32(state.pos[:, a])
        sel &= ~((c < np.float32(lo[a])) | (c >= np.float32(hi[a])))
    sc = np.float32(scale)
    for a in range(d):
        v = state.vel[sel, a].astype(np.float32) * sc
        r = np.clip(np.rint(v.astype(np.float64)), -(2.0**31), 2.0**31 - 1).astype(np.int64)
        w = (r + to_step_displacement(sys, add[a])) & 0xFFFFFFFF
        out.vel[sel, a] = np.where(w >= 1 << 31, w - (1 << 32), w).astype(np.int32)
    return out


def set_species(state, ids, species):
    """GpuEngine::set_species (md/src/engine.rs:1042-1053, reorder.wgsl:80-99)."""
    out = state.copy()
    out.species[np.asarray(ids, dtype=np.int64)] = species
    return out


def set_species_velocity(sys, state, species, v):
    """GpuEngine::set_species_velocity (md/src/engine.rs:1056-1063, md.wgsl:151-156)."""
    out = state.copy()
    sel = state.species == species
    for a in range(sys.DIM):
        out.vel[sel, a] = to_step_displacement(sys, v[a])
    return out


class IntEngine:
    """md_ref::IntEngine<F> (2D) / IntEngine3<F> (3D) on the CPU: F = f32 unless f64=True;
    `fast` selects fast.rs's path in 2D; `integer` the all-integer tables (IntEngine::integer);
    `half3` the half-shell 3D pair loop (the same kicks; the CPU baseline's form)."""

    def __init__(self, sys, state, f64=False, fast=True, integer=False, threads=1, half3=False):
        self.sys = sys
        self.n = state.n()
        self.D = sys.DIM
        self._c = sys.to_c()
        self._h = lib().oracle_engine_create(
            C.byref(self._c),
            _p(state.pos, C.c_int64),
            _p(state.vel, C.c_int32),
            _p(state.species, C.c_uint32),
            self.n,
            1 if f64 else 0,
            1 if fast else 0,
            1 if integer else 0,
            threads,
        )
        if not self._h:
            raise ValueError("oracle engine creation failed")
        if half3:
            lib().oracle_engine_set_half3(self._h, 1)
        if getattr(sys, "bonds", None):
            self.set_bonds([("fene" if t.fene else "harmonic", t.k, t.r0) for t in sys.bond_types], sys.bonds)
        if getattr(sys, "piston", None):
            drive, start, lo = sys.piston
            if lib().oracle_engine_set_piston(self._h, drive.kind, drive.speed, drive.mass, drive.force, start, lo) != 0:
                raise ValueError("the oracle refused the piston")

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_engine_destroy(self._h)
            self._h = None

    def step(self, n=1):
        lib().oracle_engine_step(self._h, n)

    def reverse(self):
        lib().oracle_engine_reverse(self._h)

    def kicks(self):
        k = np.empty((self.n, self.D), np.int32)
        pe = lib().oracle_engine_kicks(self._h, _p(k, C.c_int32))
        return k, pe

    def kicks_of(self, idx):
        """The kicks forces() gives the particles idx only (the reference loop on them)."""
        idx = np.ascontiguousarray(idx, np.uint32)
        k = np.empty((len(idx), self.D), np.int32)
        lib().oracle_engine_kicks_of(self._h, _p(idx, C.c_uint32), len(idx), _p(k, C.c_int32))
        return k

    @property
    def state(self):
        pos = np.empty((self.n, self.D), np.int64)
        vel = np.empty((self.n, self.D), np.int32)
        sp = np.empty(self.n, np.uint32)
        lib().oracle_engine_state(self._h, _p(pos, C.c_int64), _p(vel, C.c_int32), _p(sp, C.c_uint32))
        return (State if self.D == 2 else State3)(pos, vel, sp)

    def set_state(self, st):
        lib().oracle_engine_set_state(self._h, _p(st.pos, C.c_int64), _p(st.vel, C.c_int32), _p(st.species, C.c_uint32))

    def hash(self):
        return lib().oracle_engine_hash(self._h)

    def update_system(self, sys):
        """A run-time change of system (GpuEngine::update_system): the state, step counter,
        clock and ledger carry on."""
        self.sys = sys
        self._c = sys.to_c()
        lib().oracle_engine_set_system(self._h, C.byref(self._c))

    def wall_ledger(self):
        """walls::Ledger: (energy, impulse, hits), 7 slots each (2 axis + side, 6 the bath)."""
        e, p, h = (C.c_double * 7)(), (C.c_double * 7)(), (C.c_uint64 * 7)()
        lib().oracle_engine_wall_ledger(self._h, e, p, h)
        return list(e), list(p), list(h)

    def set_bonds(self, types, bonds):
        """System::with_bonds (system.rs:284-299): `types` a list of ("fene" | "harmonic", k, r0),
        `bonds` a list of (id a, id b, type index)."""
        nt = len(types)
        fene = np.array([1 if t[0] == "fene" else 0 for t in types], np.uint32)
        k = np.array([t[1] for t in types], np.float64)
        r0 = np.array([t[2] for t in types], np.float64)
        b = np.ascontiguousarray(np.array(bonds, np.uint32).reshape(-1, 3))
        lib().oracle_engine_set_bonds(self._h, _p(fene, C.c_uint32), _p(k, C.c_double), _p(r0, C.c_double), nt, _p(b, C.c_uint32), len(b))
        return self

    def compartment_ledger_fixed(self):
        """walls::CompartmentLedger in integers: (energy, impulse) in 2^-24 units and hits, arrays
        of shape (ledger slots, compartments per wall)."""
        k = lib().oracle_engine_compartment_ledger(self._h, None, None, None)
        e = np.zeros((7, k), np.int64)
        p = np.zeros((7, k), np.int64)
        h = np.zeros((7, k), np.uint64)
        lib().oracle_engine_compartment_ledger(self._h, _p(e, C.c_int64), _p(p, C.c_int64), _p(h, C.c_uint64))
        return e, p, h

    def set_piston_speed(self, u):
        """GpuEngine::set_piston_speed: the piston's velocity, u sigma/tau as a step displacement."""
        lib().oracle_engine_set_piston_speed(self._h, float(u))

    def piston(self):
        """IntEngine's piston_w (position units), piston_v (per step), piston_work (eps) and the
        gas's force on it in the last force evaluation (eps/sigma)."""
        w, v, work, f = C.c_int64(), C.c_int32(), C.c_double(), C.c_double()
        lib().oracle_engine_piston(self._h, C.byref(w), C.byref(v), C.byref(work), C.byref(f))
        return w.value, v.value, work.value, f.value

    def wall_ledger_fixed(self):
        """Every ledger event's energy change and impulse rounded to 2^-24 and summed as integers
        (in 2^-24 units), 7 slots each: the totals that do not depend on the order of events."""
        e, p = (C.c_int64 * 7)(), (C.c_int64 * 7)()
        lib().oracle_engine_wall_ledger_fixed(self._h, e, p)
        return list(e), list(p)

    def ledger(self):
        """The bath's ledger slot and the clock: (energy summed in f64 in particle order, the
        same events rounded to 2^-24 and summed as integers (in 2^-24 units), hits, clock)."""
        e, ef, h, c = C.c_double(), C.c_int64(), C.c_uint64(), C.c_uint32()
        lib().oracle_engine_ledger(self._h, C.byref(e), C.byref(ef), C.byref(h), C.byref(c))
        return e.value, ef.value, h.value, c.value

    @property
    def steps(self):
        return lib().oracle_engine_steps(self._h)

    def energy(self):
        ke, pe = C.c_double(), C.c_double()
        lib().oracle_engine_energy(self._h, C.byref(ke), C.byref(pe))
        return ke.value, pe.value


class FloatEngine:
    """md_ref::FloatEngine<f64> (2D, periodic)."""

    def __init__(self, sys, state):
        self.n = state.n()
        self._c = sys.to_c()
        self._h = lib().oracle_float_create(C.byref(self._c), _p(state.pos, C.c_int64), _p(state.vel, C.c_int32), _p(state.species, C.c_uint32), self.n)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_float_destroy(self._h)
            self._h = None

    def step(self, n=1):
        lib().oracle_float_step(self._h, n)

    def positions(self):
        out = np.empty((self.n, 2), np.float64)
        lib().oracle_float_positions(self._h, _p(out, C.c_double))
        return out

    def energy(self):
        ke, pe = C.c_double(), C.c_double()
        lib().oracle_float_energy(self._h, C.byref(ke), C.byref(pe))
        return ke.value, pe.value
