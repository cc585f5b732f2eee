"""Host-side mirror of md-core's data types (crates/md-core/src): fixed point, Pair, System,
State, System3, State3, ForceMode, and the box helpers of init.rs / three.rs.

These are plain data and exact integer/f64 host arithmetic; nothing here computes the dynamics.
"""

import ctypes as C
import math

import numpy as np

from . import _abi

ONE = 1 << 32  # fixed.rs:11
UNIT = 1.0 / ONE
DT = 0.005  # init.rs:165
SEP_LIMIT = 8 * ONE


def rust_round(x: float) -> float:
    """f64::round: half away from zero."""
    t = math.trunc(x)
    if abs(x - t) >= 0.5:
        t += math.copysign(1.0, x)
    return t


def to_fixed(x: float) -> int:
    """fixed::to_fixed (fixed.rs:21-23)."""
    return int(rust_round(x * 4294967296.0))


def to_f64(x: int) -> float:
    """fixed::to_f64 (fixed.rs:25-27)."""
    return float(x) * UNIT


def _powi(x: float, n: int) -> float:
    # Rust's f64::powi for a constant exponent: binary powering (x^6 = x^2 * (x^2)^2)
    res, have, sq = 1.0, False, x
    while n:
        if n & 1:
            res = res * sq if have else sq
            have = True
        n >>= 1
        if n:
            sq = sq * sq
    return res


class Pair:
    """md_core::Pair (pair.rs:3-57): truncated and shifted LJ."""

    __slots__ = ("eps", "sigma", "rc")

    def __init__(self, eps=1.0, sigma=1.0, rc=2.5):
        self.eps, self.sigma, self.rc = float(eps), float(sigma), float(rc)

    @staticmethod
    def lj(rc):
        return Pair(1.0, 1.0, rc)

    @staticmethod
    def wca():
        return Pair(1.0, 1.0, 2.0 ** (1.0 / 6.0))

    @staticmethod
    def none():
        return Pair(0.0, 1.0, 0.0)

    def shift(self):
        if self.eps == 0.0 or self.rc == 0.0:
            return 0.0
        s6 = _powi(self.sigma / self.rc, 6)
        return 4.0 * self.eps * s6 * (s6 - 1.0)

    def energy(self, r2):
        if r2 >= self.rc * self.rc:
            return 0.0
        s6 = _powi(self.sigma * self.sigma / r2, 3)
        return 4.0 * self.eps * s6 * (s6 - 1.0) - self.shift()

    def f_over_r(self, r2):
        if r2 >= self.rc * self.rc:
            return 0.0
        s6 = _powi(self.sigma * self.sigma / r2, 3)
        return 24.0 * self.eps * s6 * (2.0 * s6 - 1.0) / r2

    def __eq__(self, o):
        return isinstance(o, Pair) and (self.eps, self.sigma, self.rc) == (o.eps, o.sigma, o.rc)

    def __repr__(self):
        return f"Pair(eps={self.eps}, sigma={self.sigma}, rc={self.rc})"


class _SystemBase:
    DIM = 2

    def __init__(self, box_len, dt, pair, masses):
        masses = [float(m) for m in masses]
        if not (1 <= len(masses) <= _abi.MAX_SPECIES):
            raise ValueError("1 to 4 species")
        if pair.rc >= 7.9:
            raise ValueError("cutoff must be below 8 σ")
        self.box_len = [int(b) for b in box_len]
        self.dt = float(dt)
        self.masses = masses
        ns = len(masses)
        self.pairs = [Pair(pair.eps, pair.sigma, pair.rc) for _ in range(ns * ns)]
        self.gravity = [0.0] * self.DIM
        self.seed = 1
        self.pinned = 0
        self.thermostat = None
        self.walls = [None] * self.DIM
        self.membrane = None  # (axis, position, blocks mask, pore_shift, pore_width), 2D
        self.compartments = [0, 0]  # shift per axis (32 + log2 side), 2D
        self.compartments_diathermal = False
        self.bond_types = []  # Bond values
        self.bonds = []  # (id a, id b, type index)
        self.piston = None  # (Piston drive, start, min), 2D

    def species(self):
        return len(self.masses)

    def with_bonds(self, types, bonds):
        """System::with_bonds (system.rs:284-299): bond types (Bond values, at most 4) and bonds
        (id a, id b, type index), at most 4 per particle."""
        if len(types) > 4:
            raise ValueError("at most 4 bond types")
        count = {}
        for a, b, t in bonds:
            if a == b or t >= len(types):
                raise ValueError("a bond joins two particles with a known type")
            for p in (a, b):
                count[p] = count.get(p, 0) + 1
                if count[p] > 4:
                    raise ValueError(f"particle {p} has more than 4 bonds")
        self.bond_types = list(types)
        self.bonds = [tuple(int(x) for x in b) for b in bonds]
        return self

    def with_piston(self, drive, start, min):
        """System::with_piston (system.rs:274-282), 2D: the top wall of y becomes a soft piston
        starting at height `start` sigma, stopping at `min` and at the box height; y must have
        walls."""
        if self.DIM != 2:
            raise ValueError("pistons are two-dimensional")
        if self.walls[1] is None:
            raise ValueError("a piston needs walls on y")
        if not (min < start <= to_f64(self.box_len[1])):
            raise ValueError("min < start <= the box height")
        self.piston = (drive, float(start), float(min))
        return self

    def with_pair(self, a, b, pair):
        """System::with_pair (system.rs:201-207): both orders."""
        if pair.rc >= 7.9:
            raise ValueError("cutoff must be below 8 σ")
        ns = self.species()
        self.pairs[a * ns + b] = pair
        self.pairs[b * ns + a] = pair
        return self

    def with_gravity(self, g):
        self.gravity = [float(x) for x in g]
        return self

    def with_seed(self, seed):
        self.seed = int(seed)
        return self

    def with_pinned(self, s):
        self.pinned |= 1 << s
        return self

    def with_thermostat(self, t, rate):
        """System::with_thermostat (system.rs:326-333) / System3::with_thermostat (three.rs:79-83):
        an Andersen bath at kT `t`, `rate` redraws per particle per tau, keeping the species,
        region and drift of a bath already present."""
        old = self.thermostat
        self.thermostat = Thermostat(float(t), float(rate)) if old is None else Thermostat(float(t), float(rate), old.species, old.region, old.axis, old.drift)
        return self

    def pair(self, a, b):
        return self.pairs[a * self.species() + b]

    def with_walls(self, axis, lo, hi):
        """System::with_walls (system.rs:209-212): walls at 0 and L on `axis` (Wall values)."""
        self.walls[axis] = (lo, hi)
        return self

    def periodic(self, axis):
        """System::periodic (system.rs:384-386): no walls on the axis."""
        return 0 <= axis < self.DIM and self.walls[axis] is None

    def deterministic(self):
        """System::deterministic (system.rs:388-391): no heat bath and no thermal wall, so the
        dynamics is exactly reversible."""
        return self.thermostat is None and not any(w.kind == _abi.WALL_THERMAL for ws in self.walls if ws for w in ws)

    def has_soft_walls(self):
        """System::has_soft_walls (system.rs:393-395)."""
        return any(w.kind == _abi.WALL_SOFT for ws in self.walls if ws for w in ws)

    def rc_max(self):
        return max(p.rc for p in self.pairs)

    def box_f64(self):
        return [to_f64(b) for b in self.box_len]

    def volume(self):
        v = 1.0
        for b in self.box_f64():
            v *= b
        return v

    area = volume

    def kick_coeff(self, s):
        if (self.pinned >> s) & 1:
            return 0.0
        return self.dt * self.dt / self.masses[s] * 4294967296.0

    def velocity(self, v):
        return float(v) * UNIT / self.dt

    def to_step_displacement(self, v):
        return int(rust_round(v * self.dt * 4294967296.0))

    def cells_for(self, r):
        """System::cells_for (system.rs:438-444 / three.rs:151-157)."""
        b = self.box_f64()
        margin = 1e-3 + 1e-6 * max(b)
        c = [int(math.floor(l / (r + margin))) for l in b]
        if min(c) < 3:
            raise ValueError(f"box too small for radius {r}: {c} cells")
        return c

    def to_c(self) -> _abi.gbmd_system:
        s = _abi.gbmd_system()
        s.dim = self.DIM
        s.nspecies = self.species()
        for a in range(self.DIM):
            s.box_len[a] = self.box_len[a]
        s.dt = self.dt
        for k, m in enumerate(self.masses):
            s.masses[k] = m
        for k, p in enumerate(self.pairs):
            s.pairs[k].eps, s.pairs[k].sigma, s.pairs[k].rc = p.eps, p.sigma, p.rc
        for a in range(self.DIM):
            s.gravity[a] = self.gravity[a]
        s.seed = self.seed
        s.periodic = sum(1 << a for a in range(self.DIM) if self.walls[a] is None)
        for a, ws in enumerate(self.walls):
            for side, w in enumerate(ws or ()):
                s.wall_kind[a][side] = w.kind
                s.wall_t[a][side] = w.t
        if self.DIM == 2:
            s.compartments[0], s.compartments[1] = self.compartments
            s.compartments_diathermal = 1 if self.compartments_diathermal else 0
        if self.membrane is not None:
            s.membrane = 1
            s.membrane_axis, s.membrane_position, s.membrane_blocks, s.membrane_pore_shift, s.membrane_pore_width = self.membrane
        s.pinned = self.pinned
        th = self.thermostat
        if th is not None:
            s.bath = 1
            s.bath_species = th.species & 0xFFFFFFFF
            s.bath_axis = th.axis
            s.bath_t, s.bath_rate, s.bath_drift = th.t, th.rate, th.drift
            s.bath_region[0], s.bath_region[1] = th.region
        return s


class Bond:
    """md_core::BondType (system.rs:70-96): Bond.harmonic(k, r0), U = k (r - r0)^2 / 2;
    Bond.fene(k, r0), U = -k r0^2 ln(1 - (r / r0)^2) / 2; Bond.kremer_grest() = fene(30, 1.5)."""

    def __init__(self, fene, k, r0):
        self.fene, self.k, self.r0 = bool(fene), float(k), float(r0)

    @staticmethod
    def harmonic(k, r0):
        return Bond(False, k, r0)

    @staticmethod
    def fene_bond(k, r0):
        return Bond(True, k, r0)

    @staticmethod
    def kremer_grest():
        return Bond(True, 30.0, 1.5)

    def __eq__(self, o):
        return isinstance(o, Bond) and (self.fene, self.k, self.r0) == (o.fene, o.k, o.r0)

    def __repr__(self):
        return f"Bond.{'fene_bond' if self.fene else 'harmonic'}({self.k}, {self.r0})"


def chains(sys, chains, length, bond):
    """init::chains (md-core/src/init.rs:196-217): `chains` straight chains of `length` beads,
    `bond` sigma apart, laid out in rows 1 sigma clear of the box edges; returns the positions
    (id order) and the bonds (id a, id b, type 0)."""
    b = [to_f64(sys.box_len[0]), to_f64(sys.box_len[1])]
    per_row = max(int(math.floor((b[0] - 2.0) / (length * bond + 1.0))), 1)
    rows = -(-chains // per_row)
    dy = (b[1] - 2.0) / rows
    if dy < 1.0:
        raise ValueError(f"box too small for {chains} chains of {length}")
    pos, bonds = [], []
    for c in range(chains):
        row, col = c // per_row, c % per_row
        x0 = 1.0 + col * (length * bond + 1.0)
        y = 1.0 + (row + 0.5) * dy
        for k in range(length):
            i = len(pos)
            pos.append([to_fixed(x0 + k * bond), to_fixed(y)])
            if k > 0:
                bonds.append((i - 1, i, 0))
    return np.array(pos, np.int64), bonds


class Piston:
    """md_core::PistonDrive (system.rs:100-107): Piston.speed(u), moved at u sigma/tau (positive
    opens the box); Piston.free(mass, force), moved by the gas and a constant force pushing down
    (eps/sigma)."""

    SPEED, FREE = 1, 2

    def __init__(self, kind, speed=0.0, mass=0.0, force=0.0):
        self.kind, self.speed, self.mass, self.force = int(kind), float(speed), float(mass), float(force)

    @classmethod
    def speed_drive(cls, u):
        return cls(cls.SPEED, speed=u)

    @classmethod
    def free(cls, mass, force):
        return cls(cls.FREE, mass=mass, force=force)

    def __repr__(self):
        return f"Piston.speed_drive({self.speed})" if self.kind == self.SPEED else f"Piston.free({self.mass}, {self.force})"


class Wall:
    """md_core::Wall (walls.rs): Wall.hard(), Wall.soft(), Wall.thermal(t)."""

    def __init__(self, kind, t=0.0):
        self.kind, self.t = int(kind), float(t)

    @classmethod
    def hard(cls):
        return cls(_abi.WALL_HARD)

    @classmethod
    def soft(cls):
        return cls(_abi.WALL_SOFT)

    @classmethod
    def thermal(cls, t):
        return cls(_abi.WALL_THERMAL, t)

    def __eq__(self, o):
        return isinstance(o, Wall) and (self.kind, self.t) == (o.kind, o.t)

    def __repr__(self):
        return {1: "Wall.hard()", 2: "Wall.soft()"}.get(self.kind, f"Wall.thermal({self.t})")


class Thermostat:
    """md_core::Thermostat (system.rs:156-175); in 3D three::Bath (species only)."""

    def __init__(self, t, rate, species=0xFFFFFFFF, region=(-(1 << 63), (1 << 63) - 1), axis=0, drift=0.0):
        self.t, self.rate, self.species = float(t), float(rate), int(species)
        self.region, self.axis, self.drift = (int(region[0]), int(region[1])), int(axis), float(drift)

    def acts_on(self, s, p):
        """Thermostat::acts_on (system.rs:172-174)."""
        return bool(self.species & (1 << s)) and self.region[0] <= p[self.axis] < self.region[1]


class System(_SystemBase):
    """md_core::System (system.rs:26-64), periodic LJ subset."""

    DIM = 2

    def with_compartments(self, axis, log2_sigma):
        """System::with_compartments (system.rs:233-241): `axis` (with walls) split into boxes of
        2^log2_sigma sigma."""
        shift = 32 + log2_sigma
        if self.walls[axis] is None:
            raise ValueError("compartments need walls on their axis")
        if self.box_len[axis] % (1 << shift):
            raise ValueError("box must be a whole number of compartments")
        self.compartments[axis] = shift
        return self

    def with_diathermal_compartments(self):
        """System::with_diathermal_compartments (system.rs:222-226)."""
        self.compartments_diathermal = True
        return self

    def compartment_counts(self):
        """System::compartment_counts (system.rs:247-251)."""
        return [1 if self.compartments[a] == 0 else self.box_len[a] >> self.compartments[a] for a in range(2)]

    def compartment_of(self, p):
        """System::compartment_of (system.rs:253-257)."""
        return [0 if self.compartments[a] == 0 else int(p[a]) >> self.compartments[a] for a in range(2)]

    def with_membrane(self, axis, position_sigma, blocked):
        """System::with_membrane (system.rs:259-265): a membrane across walled `axis` at
        `position_sigma` that reflects the species in `blocked`."""
        if self.walls[axis] is None:
            raise ValueError("a membrane needs walls on its axis")
        mask = 0
        for b in blocked:
            mask |= 1 << b
        self.membrane = (axis, to_fixed(position_sigma), mask, 0, 0)
        return self

    def with_pores(self, log2_period, width):
        """System::with_pores (system.rs:267-274): openings `width` sigma wide every
        2^log2_period sigma along the membrane."""
        if self.membrane is None:
            raise ValueError("add a membrane first")
        a, pos, mask, _, _ = self.membrane
        self.membrane = (a, pos, mask, 32 + log2_period, to_fixed(width))
        return self

    def with_fan(self, species, x0, x1, drift):
        """System::with_fan (system.rs:335-344): the bath acts on `species` (a bitmask) with
        x0 <= x < x1 (sigma), around a mean x velocity `drift`."""
        if self.thermostat is None:
            raise ValueError("a fan is a thermostat with a region: add the thermostat first")
        th = self.thermostat
        self.thermostat = Thermostat(th.t, th.rate, species, (to_fixed(x0), to_fixed(x1)), 0, drift)
        return self

    def with_bath_layer(self, y0, y1):
        """System::with_bath_layer (system.rs:346-353): the bath acts on y0 <= y < y1 (sigma)."""
        if self.thermostat is None:
            raise ValueError("a bath layer is a thermostat with a region: add the thermostat first")
        th = self.thermostat
        self.thermostat = Thermostat(th.t, th.rate, th.species, (to_fixed(y0), to_fixed(y1)), 1, th.drift)
        return self


class System3(_SystemBase):
    """md_core::three::System3 (three.rs:13-31), periodic LJ subset."""

    DIM = 3


class _StateBase:
    DIM = 2

    def __init__(self, pos, vel, species):
        self.pos = np.ascontiguousarray(pos, dtype=np.int64).reshape(-1, self.DIM)
        self.vel = np.ascontiguousarray(vel, dtype=np.int32).reshape(-1, self.DIM)
        self.species = np.ascontiguousarray(species, dtype=np.uint32).reshape(-1)
        if not (len(self.pos) == len(self.vel) == len(self.species)):
            raise ValueError("pos, vel and species must have the same length")

    def n(self):
        return len(self.species)

    def copy(self):
        return type(self)(self.pos.copy(), self.vel.copy(), self.species.copy())

    def hash(self):
        """FNV-1a over every bit, in storage order (system.rs:460-477 / three.rs:281-297)."""
        P = C.POINTER
        return int(
            _abi.lib().gbmd_hash_state(
                self.DIM,
                self.pos.ctypes.data_as(P(C.c_int64)),
                self.vel.ctypes.data_as(P(C.c_int32)),
                self.species.ctypes.data_as(P(C.c_uint32)),
                self.n(),
            )
        )

    def permuted(self, perm):
        """Particle perm[k] of self becomes particle k (system.rs:480-486)."""
        perm = np.asarray(perm)
        return type(self)(self.pos[perm], self.vel[perm], self.species[perm])

    def unpermuted(self, perm):
        perm = np.asarray(perm)
        out = self.copy()
        out.pos[perm] = self.pos
        out.vel[perm] = self.vel
        out.species[perm] = self.species
        return out

    def velocity_sum(self):
        return [int(x) for x in self.vel.astype(np.int64).sum(axis=0)]

    def flip_bit(self, particle, axis, bit):
        self.pos[particle, axis] ^= np.int64(1) << np.int64(bit)

    def position_difference(self, other, sys):
        """Particles whose positions differ, and the largest difference in σ (system.rs:523-536)."""
        differ = np.any(self.pos != other.pos, axis=1)
        mx = 0.0
        for a in range(self.DIM):
            l = sys.box_len[a]
            d = other.pos[:, a] - self.pos[:, a]
            half = l // 2
            d = np.where(d >= half, d - l, np.where(d < -half, d + l, d))
            if differ.any():
                mx = max(mx, float(np.abs(d[differ]).max()) * UNIT)
        return int(differ.sum()), mx

    def __eq__(self, o):
        return (
            type(self) is type(o)
            and np.array_equal(self.pos, o.pos)
            and np.array_equal(self.vel, o.vel)
            and np.array_equal(self.species, o.species)
        )


class State(_StateBase):
    """md_core::State (system.rs:447-537)."""

    DIM = 2


class State3(_StateBase):
    """md_core::three::State3 (three.rs:267-309)."""

    DIM = 3


class ForceMode:
    """md::ForceMode (engine.rs:102-142): CellList or Verlet { skin, cap }."""

    VERLET_MIN_N = 24_000

    def __init__(self, kind, skin=0.0, cap=0):
        self.kind, self.skin, self.cap = kind, float(skin), int(cap)

    @staticmethod
    def cell_list():
        return ForceMode("cells")

    @staticmethod
    def verlet_with_skin(sys, n, skin, cap=0):
        """cap 0 sizes the list like verlet_with_skin / verlet3_with_skin, without the
        128 MiB single-binding clamp."""
        return ForceMode("verlet", skin, cap)

    @staticmethod
    def verlet_for(sys, n):
        return ForceMode.verlet_with_skin(sys, n, 0.4)

    @staticmethod
    def auto(sys, n):
        if sys.DIM == 2 and n < ForceMode.VERLET_MIN_N:
            return ForceMode.cell_list()
        return ForceMode.verlet_for(sys, n)

    def __repr__(self):
        return f"ForceMode({self.kind}, skin={self.skin}, cap={self.cap})"


def box_for(n, density, aspect=1.0):
    """init::box_for (init.rs:15-19)."""
    area = n / density
    ly = math.sqrt(area / aspect)
    return [to_fixed(ly * aspect), to_fixed(ly)]


def cube_for(n, density):
    """three::cube_for (three.rs:312-315)."""
    l = to_fixed(math.cbrt(n / density))
    return [l, l, l]


def fcc_cells(n, box_len):
    """three::fcc_cells (three.rs:346-355)."""
    b = [to_f64(x) for x in box_len]
    a = math.cbrt(b[0] * b[1] * b[2] * 4.0 / n)
    c = [max(int(rust_round(l / a)), 1) for l in b]
    while 4 * c[0] * c[1] * c[2] < n:
        k = 0
        for x in (1, 2):
            if b[x] / c[x] > b[k] / c[k]:
                k = x
        c[k] += 1
    return c
