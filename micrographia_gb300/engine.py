"""The engines: GpuEngine (2D) and GpuEngine3 (3D) over the C ABI of include/gbmd.h.

Their methods mirror md::GpuEngine (crates/md/src/engine.rs:598-1098) and md::GpuEngine3
(engine3.rs:334-648): construction from (System, State) with a ForceMode, asynchronous `step`,
`reverse`, `kicks`, `read_state` (id order), `upload`, `flip_bit`, `read_list_stats`,
`read_ledger`, the page commands (`kick_region`, `set_species`, `set_species_velocity`,
`sort_now`) and `update_system`, plus the CPU twins' `energy` (int_engine.rs:433-446) and the new
FP64 instruments (`observe`), and the Observer's density grid (`observe_grid`, observe.rs:26-130).
"""

import ctypes as C

import numpy as np

from . import _abi
from .core import ForceMode, State, State3
from .observe import Reading

P = C.POINTER


def _ptr(a, t):
    return a.ctypes.data_as(P(t))


def _options(mode: ForceMode, threads=0, block_steps=0, rescale_every=0, rescale_t=0.0, arith=_abi.ARITH_F32, device=0, flags=0):
    o = _abi.gbmd_options()
    o.device = device
    o.flags = flags
    if mode is None:
        o.mode = _abi.MODE_AUTO
    elif mode.kind == "cells":
        o.mode = _abi.MODE_CELLS
    else:
        o.mode = _abi.MODE_VERLET
        o.skin = mode.skin
        o.cap = mode.cap
    o.arith = arith
    o.threads = threads
    o.block_steps = block_steps
    o.rescale_every = rescale_every
    o.rescale_t = rescale_t
    return o


class _Engine:
    DIM = 2
    STATE = State

    def __init__(self, sys, state=None, mode=None, *, init=None, threads=0, block_steps=0, rescale_every=0, rescale_t=0.0, device=0,
                 arith=_abi.ARITH_F32, flags=0):
        """Create from (sys, state), or from a device-side seeded init (`init` = gbmd_init).
        `arith`: ARITH_F32 (f32 pair chain, per-pair integer kicks) or ARITH_INT (all-integer
        tables, IntEngine::integer, int_engine.rs:94-98). `flags`: gbmd_options.flags
        (FLAG_WHOLE_CELLS, build_lanes_flag(s)), list-build variants for comparisons."""
        if sys.DIM != self.DIM:
            raise ValueError(f"{type(self).__name__} needs a {self.DIM}D system")
        self.sys = sys
        self._lib = _abi.lib()
        self._csys = sys.to_c()
        self._opts = _options(mode, threads, block_steps, rescale_every, rescale_t, arith=arith, device=device, flags=flags)
        h = C.c_void_p()
        if init is not None:
            _abi.check(self._lib.gbmd_create_seeded(C.byref(self._csys), C.byref(init), C.byref(self._opts), C.byref(h)))
            self.n = init.n
        else:
            self.n = state.n()
            _abi.check(
                self._lib.gbmd_create(
                    C.byref(self._csys),
                    _ptr(state.pos, C.c_int64),
                    _ptr(state.vel, C.c_int32),
                    _ptr(state.species, C.c_uint32),
                    self.n,
                    C.byref(self._opts),
                    C.byref(h),
                )
            )
        self._h = h
        if getattr(sys, "bonds", None):
            self.set_bonds(sys.bond_types, sys.bonds)
        if getattr(sys, "piston", None):
            self.set_piston(*sys.piston)

    # -- lifecycle
    def close(self):
        if getattr(self, "_h", None):
            self._lib.gbmd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- stepping
    def step(self, steps=1):
        _abi.check(self._lib.gbmd_step(self._h, int(steps)))

    def wait(self):
        _abi.check(self._lib.gbmd_sync(self._h))

    sync = wait

    def reverse(self):
        _abi.check(self._lib.gbmd_reverse(self._h))

    # -- state
    def read_state(self):
        pos = np.empty((self.n, self.DIM), np.int64)
        vel = np.empty((self.n, self.DIM), np.int32)
        sp = np.empty(self.n, np.uint32)
        _abi.check(self._lib.gbmd_read_state(self._h, _ptr(pos, C.c_int64), _ptr(vel, C.c_int32), _ptr(sp, C.c_uint32)))
        return self.STATE(pos, vel, sp)

    def read_positions(self):
        """GpuEngine::read_positions (engine.rs:1085-1088): positions in id order."""
        pos = np.empty((self.n, self.DIM), np.int64)
        _abi.check(self._lib.gbmd_read_state(self._h, _ptr(pos, C.c_int64), None, None))
        return pos

    def read_potential(self):
        """GpuEngine3::read_potential (engine3.rs:639-643): the potential energy of the pair forces
        and soft walls at the current positions (gbmd_kicks' sum)."""
        return self.kicks()[1]

    def upload(self, state):
        if state.n() != self.n:
            raise ValueError("upload needs the same number of particles")
        _abi.check(
            self._lib.gbmd_upload(self._h, _ptr(state.pos, C.c_int64), _ptr(state.vel, C.c_int32), _ptr(state.species, C.c_uint32))
        )

    def kicks(self):
        k = np.empty((self.n, self.DIM), np.int32)
        pe = C.c_double()
        _abi.check(self._lib.gbmd_kicks(self._h, _ptr(k, C.c_int32), C.byref(pe)))
        return k, pe.value

    def snapshot(self):
        """The engine's state and counters as snapshot bytes (micrographia_gb300.snapshot)."""
        size = self._lib.gbmd_snapshot_bytes(self.DIM, self.n)
        buf = (C.c_char * size)()
        written = C.c_size_t()
        _abi.check(self._lib.gbmd_snapshot(self._h, buf, size, C.byref(written)))
        return bytes(buf)

    def restore(self, snap):
        """Resume from snapshot bytes of the same system (GbmdError if corrupted or mismatched)."""
        buf = C.create_string_buffer(bytes(snap), len(snap))
        _abi.check(self._lib.gbmd_restore(self._h, buf, len(snap)))

    def kicks_f64(self):
        """The kicks of IntEngine<f64> (f64 pair chain), the accuracy reference."""
        k = np.empty((self.n, self.DIM), np.int32)
        pe = C.c_double()
        _abi.check(self._lib.gbmd_kicks_f64(self._h, _ptr(k, C.c_int32), C.byref(pe)))
        return k, pe.value

    def flip_bit(self, particle, axis, bit):
        _abi.check(self._lib.gbmd_flip_bit(self._h, particle, axis, bit))

    # page commands and run-time changes (md::GpuEngine, crates/md/src/engine.rs:895-1063)
    def kick_region(self, lo, hi, scale, add):
        """Unpinned particles inside [lo, hi) (sigma): v <- rint(v * scale) + add (sigma/tau)."""
        arr = lambda v: (C.c_double * self.DIM)(*[float(x) for x in v])
        _abi.check(self._lib.gbmd_kick_region(self._h, arr(lo), arr(hi), float(scale), arr(add)))

    def set_species(self, ids, species):
        ids = np.ascontiguousarray(ids, dtype=np.uint32)
        _abi.check(self._lib.gbmd_set_species(self._h, _ptr(ids, C.c_uint32), int(ids.size), int(species)))

    def set_species_velocity(self, species, v):
        _abi.check(self._lib.gbmd_set_species_velocity(self._h, int(species), (C.c_double * self.DIM)(*[float(x) for x in v])))

    def sort_now(self):
        _abi.check(self._lib.gbmd_sort_now(self._h))

    def set_bonds(self, types, bonds):
        """System::with_bonds (system.rs:284-299), 2D: `types` Bond values, `bonds` (id a, id b,
        type index) triples; replaces the engine's bonds (none: an empty list)."""
        nt = len(types)
        tarr = (_abi.gbmd_bond_type * max(nt, 1))()
        for q, t in enumerate(types):
            tarr[q].kind = _abi.BOND_FENE if t.fene else _abi.BOND_HARMONIC
            tarr[q].k, tarr[q].r0 = t.k, t.r0
        b = np.ascontiguousarray(np.array(bonds, np.uint32).reshape(-1, 3))
        _abi.check(self._lib.gbmd_set_bonds(self._h, tarr, nt, _ptr(b, C.c_uint32), len(b)))

    def set_piston(self, drive, start, min):
        """System::with_piston (system.rs:274-282), 2D: a Piston drive (None removes the piston),
        the starting height and the lower stop in sigma; the upper stop is the box height."""
        p = _abi.gbmd_piston()
        if drive is not None:
            p.drive, p.speed, p.mass, p.force = drive.kind, drive.speed, drive.mass, drive.force
            p.start, p.min = float(start), float(min)
        _abi.check(self._lib.gbmd_set_piston(self._h, C.byref(p)))

    def piston(self):
        """The piston's height (position units), velocity (position units per step) and the gas's
        work on it (eps): IntEngine's piston_w, piston_v, piston_work."""
        w, v, work = C.c_int64(), C.c_int32(), C.c_double()
        _abi.check(self._lib.gbmd_read_piston(self._h, C.byref(w), C.byref(v), C.byref(work), None))
        return w.value, v.value, work.value

    def read_piston(self):
        """GpuEngine::read_piston (engine.rs:958-961): (height sigma, velocity sigma/tau, the gas's
        force on it in the last step eps/sigma, the gas's work on it eps)."""
        w, v, work, f = C.c_int64(), C.c_int32(), C.c_double(), C.c_double()
        _abi.check(self._lib.gbmd_read_piston(self._h, C.byref(w), C.byref(v), C.byref(work), C.byref(f)))
        return w.value / 4294967296.0, v.value / 4294967296.0 / self.sys.dt, f.value, work.value

    def set_piston_speed(self, u):
        """GpuEngine::set_piston_speed (engine.rs:936-939): sigma/tau, positive opens the box."""
        _abi.check(self._lib.gbmd_set_piston_speed(self._h, float(u)))

    def add_bond(self, a, b, ty):
        """GpuEngine::add_bond (engine.rs:999-1012): whether the bond was added."""
        done = C.c_int32()
        _abi.check(self._lib.gbmd_add_bond(self._h, int(a), int(b), int(ty), C.byref(done)))
        return bool(done.value)

    def remove_bond(self, a, b):
        """GpuEngine::remove_bond (engine.rs:976-985): whether there was such a bond."""
        done = C.c_int32()
        _abi.check(self._lib.gbmd_remove_bond(self._h, int(a), int(b), C.byref(done)))
        return bool(done.value)

    def flip_species_bit(self, species_mask, axis, bit):
        """GpuEngine::flip_species_bit (engine.rs:1014-1024)."""
        _abi.check(self._lib.gbmd_flip_species_bit(self._h, int(species_mask), int(axis), int(bit)))

    def update_system(self, sys):
        """Replace interactions, masses, gravity, pinned species or dt (same box and species
        count; no cutoff above the engine's largest)."""
        if sys.DIM != self.DIM:
            raise ValueError("update_system keeps the dimension")
        csys = sys.to_c()
        _abi.check(self._lib.gbmd_update_system(self._h, C.byref(csys)))
        self.sys = sys
        self._csys = csys

    def energy(self):
        ke, pe = C.c_double(), C.c_double()
        _abi.check(self._lib.gbmd_energy(self._h, C.byref(ke), C.byref(pe)))
        return ke.value, pe.value

    def observe(self, rdf_bins=0, rdf_rmax=5.0, profile_bins=0, profile_axis=0):
        """One frame: (gbmd_frame, rdf counts or None, profile counts or None)."""
        f = _abi.gbmd_frame()
        rdf = np.zeros(rdf_bins, np.uint64) if rdf_bins else None
        prof = np.zeros(profile_bins, np.uint64) if profile_bins else None
        _abi.check(
            self._lib.gbmd_observe(
                self._h,
                C.byref(f),
                _ptr(rdf, C.c_uint64) if rdf is not None else None,
                rdf_bins,
                rdf_rmax,
                _ptr(prof, C.c_uint64) if prof is not None else None,
                profile_bins,
                profile_axis,
            )
        )
        return f, rdf, prof

    def observe_grid(self, grid, marked):
        """Observer::read (observe.rs:86-97): a Reading of the gx x gy density grid, all particles
        and the `marked` species, with the half-step kinetic energy."""
        gx, gy = int(grid[0]), int(grid[1])
        all_ = np.zeros(gx * gy, np.uint32)
        mk = np.zeros(gx * gy, np.uint32)
        ke = C.c_double()
        _abi.check(self._lib.gbmd_observe_grid(self._h, gx, gy, int(marked), _ptr(all_, C.c_uint32), _ptr(mk, C.c_uint32), C.byref(ke)))
        return Reading(all_, mk, ke.value)

    def read_kinetic(self):
        """GpuEngine3::read_kinetic (engine3.rs:626-630): per-particle kinetic energies from the
        half-step velocities and the species, in id order."""
        ke = np.empty(self.n, np.float64)
        sp = np.empty(self.n, np.uint32)
        _abi.check(self._lib.gbmd_read_kinetic(self._h, _ptr(ke, C.c_double), _ptr(sp, C.c_uint32), None))
        return ke, sp

    def read_kinetic_total(self):
        """GpuEngine3::read_kinetic_total (engine3.rs:632-637)."""
        t = C.c_double()
        _abi.check(self._lib.gbmd_read_kinetic(self._h, None, None, C.byref(t)))
        return t.value

    def read_compartment_ledger(self):
        """GpuEngine::read_compartment_ledger (engine.rs:455-470): (energy, impulse, hits), arrays of
        shape (ledger slots, compartments per wall), each event rounded to 2^-24."""
        pw = C.c_uint32()
        _abi.check(self._lib.gbmd_read_compartment_ledger(self._h, 0, None, None, None, C.byref(pw)))
        k = pw.value
        e = np.zeros((_abi.LEDGER_SLOTS, k), np.float64)
        p = np.zeros((_abi.LEDGER_SLOTS, k), np.float64)
        h = np.zeros((_abi.LEDGER_SLOTS, k), np.uint64)
        _abi.check(self._lib.gbmd_read_compartment_ledger(self._h, k, _ptr(e, C.c_double), _ptr(p, C.c_double), _ptr(h, C.c_uint64), None))
        return e, p, h

    def read_ledger(self):
        """GpuEngine::read_ledger: (energy, impulse, hits), one entry per ledger slot: the walls'
        (2 axis + side) and the heat bath's (_abi.LEDGER_BATH), each event rounded to 2^-24."""
        e = (C.c_double * _abi.LEDGER_SLOTS)()
        p = (C.c_double * _abi.LEDGER_SLOTS)()
        h = (C.c_uint64 * _abi.LEDGER_SLOTS)()
        _abi.check(self._lib.gbmd_read_ledger(self._h, e, p, h))
        return list(e), list(p), list(h)

    def read_list_stats(self):
        r, o = C.c_uint32(), C.c_int32()
        _abi.check(self._lib.gbmd_list_stats(self._h, C.byref(r), C.byref(o)))
        return r.value, bool(o.value)

    def state_hash(self):
        h = C.c_uint64()
        _abi.check(self._lib.gbmd_state_hash(self._h, C.byref(h)))
        return h.value

    @property
    def steps(self):
        s, c = C.c_int64(), C.c_uint32()
        _abi.check(self._lib.gbmd_counters(self._h, C.byref(s), C.byref(c)))
        return s.value

    def stream(self):
        s = C.c_void_p()
        _abi.check(self._lib.gbmd_stream(self._h, C.byref(s)))
        return s.value

    def time_phases(self, steps):
        """`steps` steps as individual launches with CUDA events around each phase:
        (mean ms of one force step, mean ms of one list rebuild, rebuilds)."""
        f, r, n = C.c_double(), C.c_double(), C.c_uint32()
        _abi.check(self._lib.gbmd_time_phases(self._h, steps, C.byref(f), C.byref(r), C.byref(n)))
        return f.value, r.value, n.value

    def time_loop(self, steps):
        """At least `steps` steps by direct launches of the persistent step loop (small systems):
        (steps taken, mean ms per step inside the loop launches, loop launches)."""
        t, ms, n = C.c_uint32(), C.c_double(), C.c_uint32()
        _abi.check(self._lib.gbmd_time_loop(self._h, steps, C.byref(t), C.byref(ms), C.byref(n)))
        return t.value, ms.value, n.value

    def time_thermostat(self, reps):
        """The velocity-rescale thermostat's kernels run `reps` times by direct launches (each
        rescales the velocities, as a rescale step does): the mean milliseconds."""
        ms = C.c_double()
        _abi.check(self._lib.gbmd_time_thermostat(self._h, reps, C.byref(ms)))
        return ms.value

    def launch_count(self):
        c = C.c_uint64()
        _abi.check(self._lib.gbmd_launch_count(self._h, C.byref(c)))
        return c.value

    # -- introspection for parity tests
    def debug_bin(self, cells):
        cells = (C.c_uint32 * 3)(*(list(cells) + [1] * (3 - len(cells))))
        ncell = int(np.prod([cells[a] for a in range(self.DIM)]))
        keys = np.empty(self.n, np.uint32)
        start = np.empty(ncell + 1, np.uint32)
        items = np.empty(self.n, np.uint32)
        order = np.empty(self.n, np.uint32)
        _abi.check(
            self._lib.gbmd_debug_bin(
                self._h, cells, _ptr(keys, C.c_uint32), _ptr(start, C.c_uint32), _ptr(items, C.c_uint32), _ptr(order, C.c_uint32)
            )
        )
        return keys, start, items, order

    def debug_barrier_timeout(self, blocks=4):
        """Raw status of gbmd_debug_barrier_timeout (the step loop's barrier running out)."""
        return self._lib.gbmd_debug_barrier_timeout(self._h, int(blocks))

    def debug_list_flat(self, max_total=None):
        """The Verlet lists in id order, packed: (counts, offsets, neighbour ids); particle i's
        neighbours are ids[offsets[i]:offsets[i + 1]], unsorted."""
        counts = np.empty(self.n, np.uint32)
        cap = max_total or self.n * 256
        nbr = np.empty(cap, np.uint32)
        _abi.check(self._lib.gbmd_debug_list(self._h, _ptr(counts, C.c_uint32), _ptr(nbr, C.c_uint32), cap))
        offs = np.concatenate([[0], np.cumsum(counts.astype(np.int64))])
        return counts, offs, nbr

    def debug_list(self, max_total=None):
        _, offs, nbr = self.debug_list_flat(max_total)
        return [np.sort(nbr[offs[i] : offs[i + 1]]) for i in range(self.n)]


class GpuEngine(_Engine):
    """md::GpuEngine: 2D. `mode` None selects ForceMode::auto (cell list below 24 000)."""

    DIM = 2
    STATE = State

    @classmethod
    def with_mode(cls, sys, state, mode, **kw):
        return cls(sys, state, mode, **kw)


class GpuEngine3(_Engine):
    """md::GpuEngine3: 3D, Verlet lists by default (engine3.rs:337-340)."""

    DIM = 3
    STATE = State3

    def __init__(self, sys, state=None, mode=None, **kw):
        if mode is None:
            mode = ForceMode.verlet_for(sys, state.n() if state is not None else kw["init"].n)
        super().__init__(sys, state, mode, **kw)

    @classmethod
    def with_mode(cls, sys, state, mode, **kw):
        return cls(sys, state, mode, **kw)


def init_state(sys, recipe, n, t, seed, jitter=0.1, rho_liquid=0.7, rho_vapour=0.05, slab_frac=0.25):
    """Generate a seeded initial state on the device (gbmd_init_state) and return it."""
    spec = make_init(recipe, n, t, seed, jitter, rho_liquid, rho_vapour, slab_frac)
    D = sys.DIM
    pos = np.empty((n, D), np.int64)
    vel = np.empty((n, D), np.int32)
    sp = np.empty(n, np.uint32)
    csys = sys.to_c()
    _abi.check(
        _abi.lib().gbmd_init_state(C.byref(csys), C.byref(spec), _ptr(pos, C.c_int64), _ptr(vel, C.c_int32), _ptr(sp, C.c_uint32))
    )
    return (State if D == 2 else State3)(pos, vel, sp)


def make_init(recipe, n, t, seed, jitter=0.1, rho_liquid=0.7, rho_vapour=0.05, slab_frac=0.25):
    spec = _abi.gbmd_init()
    spec.recipe = recipe
    spec.n = n
    spec.t = t
    spec.seed = seed
    spec.jitter = jitter
    spec.rho_liquid = rho_liquid
    spec.rho_vapour = rho_vapour
    spec.slab_frac = slab_frac
    return spec


class BatchEngine:
    """Many independent periodic systems stepped together (gbmd_batch_*)."""

    def __init__(self, systems, states, mode=None, threads=0, block_steps=0, device=0, tune_skin=False, force_lanes=0):
        """With `tune_skin`, the autotuner picks the Verlet skin (the fastest of 0.3..0.7 sigma)
        and then the force lanes per particle (1, 2 or 4) on short timed runs from these states
        (mode's skin and `force_lanes` ignored); the trajectory is the same for any choice."""
        self._lib = _abi.lib()
        if len(systems) != len(states) or not systems:
            raise ValueError("one state per system")
        D = systems[0].DIM
        if any(s.DIM != D for s in systems):
            raise ValueError("a batch holds systems of one dimension")
        if any(getattr(s, "bonds", None) for s in systems):
            raise ValueError("a batch holds pair systems: bonded systems run on GpuEngine")
        self.D = D
        self.count = len(systems)
        self.sizes = [st.n() for st in states]
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.uint32)
        csys = (_abi.gbmd_system * self.count)(*[s.to_c() for s in systems])
        pos = np.ascontiguousarray(np.concatenate([st.pos for st in states]))
        vel = np.ascontiguousarray(np.concatenate([st.vel for st in states]))
        sp = np.ascontiguousarray(np.concatenate([st.species for st in states]))
        opts = _options(mode or ForceMode.verlet_for(systems[0], 0), threads, block_steps, device=device,
                        flags=(_abi.FLAG_TUNE_SKIN if tune_skin else 0) | (int(force_lanes) << 8))
        h = C.c_void_p()
        _abi.check(
            self._lib.gbmd_batch_create(
                csys,
                self.count,
                _ptr(self.offsets, C.c_uint32),
                _ptr(pos, C.c_int64),
                _ptr(vel, C.c_int32),
                _ptr(sp, C.c_uint32),
                C.byref(opts),
                C.byref(h),
            )
        )
        self._h = h

    def step(self, steps=1):
        _abi.check(self._lib.gbmd_batch_step(self._h, int(steps)))

    @property
    def skin(self):
        v = C.c_double()
        _abi.check(self._lib.gbmd_batch_skin(self._h, C.byref(v)))
        return v.value

    @property
    def force_lanes(self):
        v = C.c_uint32()
        _abi.check(self._lib.gbmd_batch_force_lanes(self._h, C.byref(v)))
        return v.value

    def read_ledger(self, k):
        """System k's ledger (energy, impulse, hits per slot), as GpuEngine.read_ledger."""
        e = (C.c_double * _abi.LEDGER_SLOTS)()
        p = (C.c_double * _abi.LEDGER_SLOTS)()
        h = (C.c_uint64 * _abi.LEDGER_SLOTS)()
        _abi.check(self._lib.gbmd_batch_read_ledger(self._h, k, e, p, h))
        return list(e), list(p), list(h)

    def wait(self):
        _abi.check(self._lib.gbmd_batch_sync(self._h))

    def read_system(self, k):
        n = self.sizes[k]
        pos = np.empty((n, self.D), np.int64)
        vel = np.empty((n, self.D), np.int32)
        sp = np.empty(n, np.uint32)
        _abi.check(self._lib.gbmd_batch_read_system(self._h, k, _ptr(pos, C.c_int64), _ptr(vel, C.c_int32), _ptr(sp, C.c_uint32)))
        return (State if self.D == 2 else State3)(pos, vel, sp)

    def read_all(self):
        """Every system's id-ordered state (one conversion for the whole batch), as a list."""
        N = int(self.offsets[-1])
        pos = np.empty((N, self.D), np.int64)
        vel = np.empty((N, self.D), np.int32)
        sp = np.empty(N, np.uint32)
        _abi.check(self._lib.gbmd_batch_read_all(self._h, _ptr(pos, C.c_int64), _ptr(vel, C.c_int32), _ptr(sp, C.c_uint32)))
        cls = State if self.D == 2 else State3
        o = self.offsets
        return [cls(pos[o[k] : o[k + 1]].copy(), vel[o[k] : o[k + 1]].copy(), sp[o[k] : o[k + 1]].copy()) for k in range(self.count)]

    def observe(self, rdf_bins=0, rdf_rmax=5.0):
        """A frame of every system (gbmd_batch_observe): a list of gbmd_frame, and the RDF counts
        as an array of shape (systems, rdf_bins) or None."""
        frames = (_abi.gbmd_frame * self.count)()
        rdf = np.zeros((self.count, rdf_bins), np.uint64) if rdf_bins else None
        _abi.check(self._lib.gbmd_batch_observe(self._h, frames, _ptr(rdf, C.c_uint64) if rdf is not None else None, rdf_bins, rdf_rmax))
        return list(frames), rdf

    def stream(self):
        s = C.c_void_p()
        _abi.check(self._lib.gbmd_batch_stream(self._h, C.byref(s)))
        return s.value

    def stats(self):
        l, r = C.c_uint64(), C.c_uint32()
        _abi.check(self._lib.gbmd_batch_stats(self._h, C.byref(l), C.byref(r)))
        return l.value, r.value

    def time_phases(self, steps):
        """`steps` steps as individual launches with CUDA events around the force launch and the
        list rebuild: (mean ms of one force step, mean ms of one rebuild, rebuilds)."""
        f, r, n = C.c_double(), C.c_double(), C.c_uint32()
        _abi.check(self._lib.gbmd_batch_time_phases(self._h, steps, C.byref(f), C.byref(r), C.byref(n)))
        return f.value, r.value, n.value

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gbmd_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """The serving loop (gbmd_serve_*): submit requests, poll frames."""

    def __init__(self, hbm_budget_bytes, max_active=64, device=0, lane_max_n=None):
        """`lane_max_n`: requests of at most this many particles are stepped together in their
        dimension's lane batch (None: the library's default, 65,536; 0: every request on an
        engine of its own)."""
        self._lib = _abi.lib()
        h = C.c_void_p()
        _abi.check(self._lib.gbmd_serve_create(int(hbm_budget_bytes), max_active, device, C.byref(h)))
        self._h = h
        self._buf = (_abi.gbmd_serve_frame * 64)()
        if lane_max_n is not None:
            _abi.check(self._lib.gbmd_serve_set_lanes(self._h, int(lane_max_n)))

    def submit(self, sys, init, steps, frame_every=100, rdf_bins=200, rdf_rmax=5.0, skin=0.3):
        if getattr(sys, "bonds", None):
            raise ValueError("the server runs pair systems: bonded systems run on GpuEngine")
        r = _abi.gbmd_serve_request()
        r.sys = sys.to_c()
        r.init = init
        r.steps = steps
        r.frame_every = frame_every
        r.rdf_bins = rdf_bins
        r.rdf_rmax = rdf_rmax
        r.skin = skin
        rid = C.c_uint64()
        _abi.check(self._lib.gbmd_serve_submit(self._h, C.byref(r), C.byref(rid)))
        return rid.value

    def poll(self):
        """Frames delivered since the last poll (copies)."""
        out = []
        while True:
            cnt = C.c_uint32()
            _abi.check(self._lib.gbmd_serve_poll(self._h, self._buf, len(self._buf), C.byref(cnt)))
            for k in range(cnt.value):
                f = _abi.gbmd_serve_frame()
                C.pointer(f)[0] = self._buf[k]
                out.append(f)
            if cnt.value < len(self._buf):
                return out

    def cancel(self, rid):
        _abi.check(self._lib.gbmd_serve_cancel(self._h, rid))

    def stats(self):
        st = _abi.gbmd_serve_stats_t()
        _abi.check(self._lib.gbmd_serve_stats(self._h, C.byref(st)))
        return st

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gbmd_serve_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
