/*
 * gbmd.h — C ABI of the GB300-native integer fixed-point Lennard-Jones MD engine.
 *
 * This is the drop-in boundary for the engine interface that micrographia's `scenarios` crate,
 * its pages and its tests drive: the method set shared by `md::GpuEngine`
 * (crates/md/src/engine.rs:598-1098), `md::GpuEngine3` (crates/md/src/engine3.rs:334-648) and
 * their CPU twins `md_ref::IntEngine<F>` (crates/md-ref/src/int_engine.rs:52-447) and
 * `md_ref::IntEngine3<F>` (crates/md-ref/src/int_engine3.rs:28-240).
 *
 * Layouts are md-core's, so a Rust `extern "C"` crate passes `State` vectors without conversion:
 *   - positions: int64 in units of 2^-32 sigma, interleaved per particle ([i64; 2] or [i64; 3]),
 *     as `md_core::State::pos` / `State3::pos` (crates/md-core/src/system.rs:447-453);
 *   - velocities: int32 displacement per step (v_{n-1/2} dt 2^32), interleaved as `State::vel`;
 *   - species: uint32 per particle.
 * All arrays handed across the ABI are in particle-id order (the order of the State given at
 * creation); the engine's own storage order is private, as in the reference (ids buffer,
 * crates/md/src/engine.rs:383-389).
 *
 * Conventions (the reference panics or returns `GpuError(String)`, crates/gpu-prims/src/context.rs:15-24):
 *   - every call returns an int status: GBMD_OK (0) or a negative GBMD_E_* code;
 *     gbmd_last_error() returns a thread-local message describing the last failure;
 *   - the caller owns host arrays, the engine owns device memory;
 *   - an engine is used from one host thread at a time; work is stream-ordered and asynchronous
 *     (gbmd_step returns before the GPU finishes; read calls wait);
 *   - no callbacks.
 */
#ifndef GBMD_H
#define GBMD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBMD_MAX_SPECIES 4 /* md_core::system::MAX_SPECIES (crates/md-core/src/system.rs:7) */

/* Status codes. */
#define GBMD_OK 0
#define GBMD_E_INVALID (-1)     /* invalid configuration or argument (the reference's assert!s) */
#define GBMD_E_NOMEM (-2)       /* device allocation failed */
#define GBMD_E_BUDGET (-3)      /* over the engine's or server's HBM budget */
#define GBMD_E_OVERFLOW (-4)    /* a neighbour list overflowed its capacity */
#define GBMD_E_NONFINITE (-5)   /* a non-finite energy or force was met */
#define GBMD_E_TIMEOUT (-6)     /* a bounded device-side wait gave up */
#define GBMD_E_CUDA (-7)        /* a CUDA runtime error */
#define GBMD_E_UNSUPPORTED (-8) /* a System feature this engine does not implement */
#define GBMD_E_NOTFOUND (-9)    /* unknown request or slot */

/* Force modes: md::ForceMode (crates/md/src/engine.rs:102-142). */
#define GBMD_MODE_AUTO 0   /* cell list below 24 000 particles in 2D, Verlet lists otherwise */
#define GBMD_MODE_CELLS 1  /* scan the 3x3(x3) neighbouring cells every step */
#define GBMD_MODE_VERLET 2 /* Verlet lists with a skin and a displacement-triggered rebuild */

/* Pair arithmetic: md::Arith (crates/md/src/engine.rs:89-100). */
#define GBMD_ARITH_F32 0 /* f32 pair forces, each pair's kick rounded to an integer */
#define GBMD_ARITH_INT 1 /* all-integer table forces (md_core::table::IntTables) */

/* md_core::Pair (crates/md-core/src/pair.rs:3-8): truncated and shifted LJ. */
typedef struct gbmd_pair {
    double eps;
    double sigma;
    double rc;
} gbmd_pair;

/*
 * The System fields the LJ path needs: md_core::System (crates/md-core/src/system.rs:26-64) and
 * md_core::three::System3 (crates/md-core/src/three.rs:13-31). `pairs` is row-major
 * [a * nspecies + b] like `System::pairs`. Walls (hard, soft, thermal) run on plain engines;
 * compartments, membranes, pistons and bonds are outside this engine, and batches and served
 * requests take periodic systems only.
 *
 * The Andersen heat bath (`bath` = 1): md_core::Thermostat (system.rs:156-175, built by
 * with_thermostat / with_fan / with_bath_layer, system.rs:326-353) in 2D and three::Bath
 * (three.rs:79-81) in 3D. After its kick, a particle of a species in `bath_species`, not pinned,
 * and (2D) with its position along `bath_axis` in [bath_region[0], bath_region[1]) is given a new
 * Maxwell velocity at bath_t with probability bath_rate * dt per step, drawn from Threefry on
 * (its id, the engine's step clock): walls::andersen (walls.rs:113-133) and three::andersen
 * (three.rs:247-265). 2D adds the fan's drift to the new x velocity. The energy the bath gives
 * is booked in ledger slot GBMD_LEDGER_BATH.
 */
typedef struct gbmd_system {
    uint32_t dim;      /* 2 or 3 */
    uint32_t nspecies; /* 1..GBMD_MAX_SPECIES */
    int64_t box_len[3];/* position units; box_len[2] unused in 2D */
    double dt;
    double masses[GBMD_MAX_SPECIES];
    gbmd_pair pairs[GBMD_MAX_SPECIES * GBMD_MAX_SPECIES];
    double gravity[3]; /* sigma/tau^2 */
    uint64_t seed;
    uint32_t periodic; /* bit a set if axis a is periodic */
    uint32_t pinned;   /* bit s set if species s is pinned */
    uint32_t bath;          /* 1: an Andersen heat bath (Some(Thermostat)); 0: none */
    uint32_t bath_species;  /* bit s set if it acts on species s (with_thermostat: all) */
    uint32_t bath_axis;     /* 2D: the axis of its region (0 x: a fan; 1 y: a bath layer) */
    uint32_t _bath_pad;
    double bath_t;          /* kT */
    double bath_rate;       /* redraws per particle per tau */
    double bath_drift;      /* 2D: mean x velocity of redrawn particles, sigma/tau */
    int64_t bath_region[2]; /* 2D: [lo, hi) along bath_axis in position units (all: INT64_MIN, INT64_MAX) */
    /* Walls on the axes whose `periodic` bit is clear (md_core::Wall, walls.rs; with_walls,
     * system.rs:209-212): wall_kind[axis][side] (side 0 at 0, 1 at L) is a GBMD_WALL_* kind,
     * wall_t[axis][side] a thermal wall's kT. A walled axis needs a kind on each side. After each
     * force step a pass adds the soft walls' kicks, applies the bath, and mirrors a particle that
     * left the box back in (walls::mirror), colliding it with the wall (IntEngine::collide,
     * int_engine.rs:363-390; int_engine3.rs:186-205). */
    uint32_t wall_kind[3][2];
    double wall_t[3][2];
    /* A semi-permeable membrane across a walled axis (md_core::Membrane, system.rs:119-141;
     * with_membrane / with_pores, system.rs:259-274), 2D: it reflects the species in
     * membrane_blocks about membrane_position - 1/2, except through pores membrane_pore_width wide
     * every 2^membrane_pore_shift position units along it (shift 0: no pores). A crossing is
     * mirrored after the force step and booked in the ledger's faces 4 and 5. */
    uint32_t membrane;      /* 1: present */
    uint32_t membrane_axis;
    uint32_t membrane_blocks;
    uint32_t membrane_pore_shift;
    int64_t membrane_position;
    int64_t membrane_pore_width;
    /* Compartments (System::with_compartments, system.rs:233-241), 2D: a walled axis split into
     * boxes of 2^(compartments[axis] - 32) sigma by hard walls (0: none); particles in different
     * boxes interact only when compartments_diathermal is 1 (CompartmentWalls, system.rs:143-153).
     * A particle that crossed into another box is mirrored back home after the force step;
     * insulating boxes are filtered from the lists and the cell-list pairs. */
    uint32_t compartments[2];
    uint32_t compartments_diathermal;
    uint32_t _compartments_pad;
} gbmd_system;

/* gbmd_system.wall_kind: md_core::Wall (walls.rs). */
#define GBMD_WALL_HARD 1    /* exact mirror, v -> -v */
#define GBMD_WALL_SOFT 2    /* WCA repulsion in the distance to the wall (walls.rs:103-111) */
#define GBMD_WALL_THERMAL 3 /* a hit draws a Maxwell-flux velocity at wall_t (walls.rs:89-101) */

/* Engine options: ForceMode + Arith + the engine's own tuning knobs. Zero-initialised is valid. */
/* gbmd_options.flags */
#define GBMD_FLAG_WHOLE_CELLS 1u /* list builds scan whole neighbour cells (no slab sub-buckets): timing comparisons */
#define GBMD_FLAG_NO_STEP_LOOP 2u /* small systems step through per-step graph nodes, not the persistent step loop: comparisons */
/* batches only: gbmd_batch_create's autotuner. It times two blocks of (at most 100) steps from the
 * given state at each skin of 0.3, 0.4, 0.5, 0.6 and 0.7 sigma (the rebuild cadence) with one force
 * lane per particle, then 2 and 4 lanes per particle (neighbours per warp) at the fastest skin, and
 * keeps the fastest; `skin` and the force lanes asked for are ignored. The trajectory depends on
 * neither (the lists hold exactly the pairs within the cutoff; integer kicks sum in any order).
 * Batches take 1, 2 or 4 force lanes (GBMD_FLAG_FORCE_LANES; others: 1). */
#define GBMD_FLAG_TUNE_SKIN 4u
/* bits 4-7 of flags: lanes per particle of the list build (1, 2, 4 or 8; 0 chooses by size) */
#define GBMD_FLAG_BUILD_LANES(s) ((uint32_t)(s) << 4)
/* bits 8-12 of flags: lanes per particle of the force step (1, 2, 4, 8 or 16; 0 chooses by size) */
#define GBMD_FLAG_FORCE_LANES(s) ((uint32_t)(s) << 8)
/* Half-shell lists (3D, one species): each pair listed once and its pair chain evaluated once,
 * its kick mirrored onto the other particle through shared-memory row windows. The trajectory is
 * the same as with full lists, bit for bit; on GB300 the full-list step is faster (the default). */
#define GBMD_FLAG_HALF_LISTS 16384u /* bit 14 */
/* 2D Verlet lists: each particle's path since the list build (the sum of |vx| + |vy| over its
 * steps) rides in its quotient record, and while it stays below what could fire the displacement
 * trigger the step skips the test (and the read of the reference position). The trigger fires at
 * the same steps either way. This flag turns the bound off: comparisons. */
#define GBMD_FLAG_NO_PATH_BOUND 32768u /* bit 15 */

typedef struct gbmd_options {
    int32_t mode;          /* GBMD_MODE_* */
    int32_t arith;         /* GBMD_ARITH_* */
    double skin;           /* Verlet skin in sigma; <= 0 selects 0.4 (ForceMode::verlet_for) */
    uint32_t cap;          /* list capacity per particle; 0 sizes it like verlet_with_skin */
    uint32_t block_steps;  /* steps per captured CUDA-graph block; 0 selects 64 */
    int32_t device;        /* CUDA device ordinal */
    uint32_t threads;      /* threads per block for the force kernel; 0 selects the tuned value */
    uint32_t rescale_every;/* velocity-rescale thermostat period in steps (0: off) */
    uint32_t flags;        /* GBMD_FLAG_* */
    double rescale_t;      /* thermostat target kT */
} gbmd_options;

typedef struct gbmd_engine gbmd_engine;

/* Observables of one frame, FP64 reductions on the device (new in this engine: the reference
 * has only f32 kinetic totals, crates/md/shaders/observe.wgsl:48-56). */
typedef struct gbmd_frame {
    uint64_t step;        /* net steps taken */
    double kinetic;       /* on-step kinetic energy (IntEngine::energy, int_engine.rs:433-446) */
    double potential;     /* potential energy: pairs, bonds, soft walls, the piston, and gravity's -m g . x */
    double virial;        /* sum over pairs of r . F = sum fr r^2 (mc/src/gibbs.rs:58-66) */
    double temperature;   /* 2 KE / (dim (N - 1)) */
    double pressure;      /* rho T + virial / (dim V) */
    double volume;
    uint32_t n;
    uint32_t dim;
} gbmd_frame;

/* ---- Engine lifecycle: GpuEngine::{new, with_mode, with_options} ---- */

/* Create an engine from a system and a state (copied to the device). `opts` may be NULL. */
int gbmd_create(const gbmd_system* sys, const int64_t* pos, const int32_t* vel,
                const uint32_t* species, uint32_t n, const gbmd_options* opts, gbmd_engine** out);
int gbmd_destroy(gbmd_engine* e);

/* ---- Stepping: GpuEngine::step (engine.rs:852-873), reverse (engine.rs:881) ---- */

/* Enqueue `steps` leapfrog steps; returns without waiting for the GPU. */
int gbmd_step(gbmd_engine* e, uint64_t steps);
/* Wait for all enqueued work; reports a deferred device error (list overflow, CUDA). */
int gbmd_sync(gbmd_engine* e);
/* Time reversal v <- -(v + kick(x) + g) (IntEngine::reverse, int_engine.rs:396-413). */
int gbmd_reverse(gbmd_engine* e);

/* ---- State I/O in id order: read_state (engine.rs:1080), upload (engine.rs:1067) ---- */

int gbmd_read_state(gbmd_engine* e, int64_t* pos, int32_t* vel, uint32_t* species);
int gbmd_upload(gbmd_engine* e, const int64_t* pos, const int32_t* vel, const uint32_t* species);
/* Integer kicks at the current positions and the pair potential energy (engine.rs:1089-1097). */
int gbmd_kicks(gbmd_engine* e, int32_t* kicks, double* potential);
/* The same kicks with the pair chain in f64 (IntEngine<f64>::forces, int_engine.rs:130-251 with
 * F = f64): the accuracy reference of the f32 path, computed on the device at full size. */
int gbmd_kicks_f64(gbmd_engine* e, int32_t* kicks, double* potential);
/* Checkpoint / resume: a binary snapshot of the dynamical state (id order) and the step counter,
 * clock and thermostat phase, with the state's FNV-1a hash. Layout (little-endian): "GBMDSNP1",
 * u32 version 1, dim, n, 0; i64 steps; u32 clock, 0; u64 thermostat phase; u64 hash; then
 * positions i64[dim n], velocities i32[dim n], species u32[n]. gbmd_restore requires the same
 * dimension and particle count and rejects a snapshot whose arrays do not match its hash; a run
 * of 2N steps equals N steps, snapshot, restore (in any engine of the same system), N steps. */
size_t gbmd_snapshot_bytes(uint32_t dim, uint32_t n);
int gbmd_snapshot(gbmd_engine* e, void* buf, size_t cap, size_t* written);
int gbmd_restore(gbmd_engine* e, const void* buf, size_t size);
/* Flip one bit of one coordinate of particle `id` (engine.rs:964, State::flip_bit). */
int gbmd_flip_bit(gbmd_engine* e, uint32_t id, uint32_t axis, uint32_t bit);
/* GpuEngine::flip_species_bit (engine.rs:1014-1024): XOR bit `bit` of coordinate `axis` of every
 * particle whose species is in the mask `species_mask`. */
int gbmd_flip_species_bit(gbmd_engine* e, uint32_t species_mask, uint32_t axis, uint32_t bit);

/* ---- Page commands and run-time changes: md::GpuEngine (crates/md/src/engine.rs:895-1063) ---- */

/* engine.rs:1026-1036 (md.wgsl:216-229, md3.wgsl:541-553): for every unpinned particle whose f32
 * position, f32(x >> 32) + f32(x & 0xffffffff) 2^-32 per axis, lies in [lo, hi) (bounds rounded
 * to f32): v <- rint(f32(v) * f32(scale)) + add on each axis, `add` a velocity in sigma/tau turned
 * into position units per step by System::to_step_displacement. lo, hi, add: `dim` entries. */
int gbmd_kick_region(gbmd_engine* e, const double* lo, const double* hi, double scale, const double* add);
/* engine.rs:1042-1053 (reorder.wgsl:80-99): the particles with these ids (any order, repeats
 * allowed) take `species`; masses and forces follow from the next step (the lists are rebuilt). */
int gbmd_set_species(gbmd_engine* e, const uint32_t* ids, uint32_t count, uint32_t species);
/* engine.rs:1056-1063 (md.wgsl:151-156): every particle of `species` gets the velocity v
 * (sigma/tau, `dim` entries, as position units per step). */
int gbmd_set_species_velocity(gbmd_engine* e, uint32_t species, const double* v);
/* engine.rs:943-947: re-sort the storage into cell order and rebuild the lists now (the
 * reference sorts into Morton order; the storage order is invisible to results either way). */
int gbmd_sort_now(gbmd_engine* e);
/* engine.rs:895-934: replace the interactions, masses, gravity, pinned species or dt at run time.
 * The dimension, box and species count stay; no cutoff may exceed the largest the engine was
 * built with (its cells and list capacity are sized by it); an all-integer engine keeps its
 * tables (pairs, masses, dt, pinned). Velocities are kept as they are (position units per step).
 * The lists are rebuilt before the next step. GBMD_E_INVALID otherwise, the engine unchanged. */
int gbmd_update_system(gbmd_engine* e, const gbmd_system* sys);
/* Bonds (md_core::BondType, system.rs:70-96; System::with_bonds, system.rs:284-299), 2D: `ntypes`
 * bond types and `nbonds` bonds, three words each (particle id a, id b, type index), at most
 * GBMD_MAX_BONDS per particle; each bond's kick is rounded on its own like a pair's
 * (IntEngine::forces, int_engine.rs:185-202), with the separation's long form beyond 8 sigma
 * (fixed.rs:63-72). Replaces the engine's bonds (nbonds 0: none), before stepping or between
 * steps. GBMD_E_UNSUPPORTED in 3D (IntEngine3 has no bonds) and with integer table forces. */
#define GBMD_MAX_BONDS 4      /* system.rs:66 */
#define GBMD_MAX_BOND_TYPES 4 /* system.rs:67 */
#define GBMD_BOND_HARMONIC 0  /* U = k (r - r0)^2 / 2 (a zero-length spring when r0 = 0) */
#define GBMD_BOND_FENE 1      /* U = -k r0^2 ln(1 - (r / r0)^2) / 2, its argument capped at 1 - 1e-6 */
typedef struct gbmd_bond_type {
    uint32_t kind; /* GBMD_BOND_* */
    uint32_t _pad;
    double k;
    double r0;
} gbmd_bond_type;
int gbmd_set_bonds(gbmd_engine* e, const gbmd_bond_type* types, uint32_t ntypes, const uint32_t* bonds, uint32_t nbonds);
/* GpuEngine::add_bond / remove_bond (engine.rs:976-1012): bond ids a and b with bond type `type`
 * (one of the types gbmd_set_bonds gave), as in a reaction, or break their bond for good; *done
 * is 1 if the bond list changed, 0 if they were already bonded (or one has GBMD_MAX_BONDS bonds,
 * or a == b) / had no bond. Between steps. */
int gbmd_add_bond(gbmd_engine* e, uint32_t a, uint32_t b, uint32_t type, int32_t* done);
int gbmd_remove_bond(gbmd_engine* e, uint32_t a, uint32_t b, int32_t* done);
/* The piston (md_core::Piston, system.rs:100-116; System::with_piston, system.rs:274-282), 2D: a
 * soft wall that replaces the top of y (the axis must have walls), starting at height `start`
 * sigma and stopping at `min` and at the box height. GBMD_PISTON_SPEED moves it at `speed`
 * sigma/tau (positive opens the box; a heat bath then draws relative to its affine flow,
 * int_engine.rs:282-286); GBMD_PISTON_FREE lets the gas move it against `force` eps/sigma pushing
 * down, with mass `mass` (walls::piston_kick, walls.rs:143-146). Each step the gas's force on it
 * is summed in 2^-16 eps/sigma units (walls.rs:140-141) and the piston moves after the particles
 * (IntEngine::move_piston, int_engine.rs:346-361); particles that pass it are mirrored below it.
 * GBMD_PISTON_NONE removes it. Set before stepping or between steps; GBMD_E_UNSUPPORTED in 3D,
 * GBMD_E_INVALID for a periodic y or bad values. */
#define GBMD_PISTON_NONE 0
#define GBMD_PISTON_SPEED 1
#define GBMD_PISTON_FREE 2
typedef struct gbmd_piston {
    uint32_t drive; /* GBMD_PISTON_* */
    uint32_t _pad;
    double speed;   /* sigma/tau (GBMD_PISTON_SPEED) */
    double mass;    /* GBMD_PISTON_FREE */
    double force;   /* eps/sigma pushing down (GBMD_PISTON_FREE) */
    double start;   /* sigma */
    double min;     /* sigma */
} gbmd_piston;
int gbmd_set_piston(gbmd_engine* e, const gbmd_piston* piston);
/* IntEngine's piston_w (height, position units), piston_v (position units per step),
 * piston_work (the gas's work on the piston, eps) and the gas's force on it in the last step
 * (eps/sigma; GpuEngine::read_piston, engine.rs:958-961). Any pointer may be NULL. */
int gbmd_read_piston(gbmd_engine* e, int64_t* height, int32_t* velocity, double* work, double* force);
/* GpuEngine::set_piston_speed (engine.rs:936-939): the piston's velocity, sigma/tau (positive
 * opens the box), as a step displacement. */
int gbmd_set_piston_speed(gbmd_engine* e, double speed);

/* ---- Observables: IntEngine::energy (int_engine.rs:433-446) and the new instruments ---- */

int gbmd_energy(gbmd_engine* e, double* kinetic, double* potential);
/* GpuEngine3::read_kinetic / read_kinetic_total (engine3.rs:618-637) and
 * Observer::read_kinetic_energies (observe.rs:99-117): each particle's kinetic energy 1/2 m |v|^2
 * from its half-step velocity (0 for a pinned species), and its species, in id order, and their
 * total (f64, where the reference reads f32; any pointer may be NULL). */
int gbmd_read_kinetic(gbmd_engine* e, double* kinetic, uint32_t* species, double* total);
/* One frame of instruments. `rdf` (may be NULL) receives `rdf_bins` integer pair counts of
 * unordered pairs with floor(r * rdf_bins / rdf_rmax) = k; `profile` (may be NULL) receives
 * `profile_bins` particle counts along `profile_axis`. */
int gbmd_observe(gbmd_engine* e, gbmd_frame* frame, uint64_t* rdf, uint32_t rdf_bins,
                 double rdf_rmax, uint64_t* profile, uint32_t profile_bins, uint32_t profile_axis);
/* gbmd_observe in two halves, for callers that overlap frames with other work: _begin enqueues
 * the frame's kernels and copies on the engine's stream and returns at once (0 bins: no RDF /
 * no profile); _end waits for them (at once if an event recorded after _begin has completed)
 * and fills `frame`, `rdf` (rdf_bins counts) and `profile`. One frame in flight per engine. */
int gbmd_observe_begin(gbmd_engine* e, uint32_t rdf_bins, double rdf_rmax, uint32_t profile_bins, uint32_t profile_axis);
int gbmd_observe_end(gbmd_engine* e, gbmd_frame* frame, uint64_t* rdf, uint64_t* profile);
/* Observer::read (crates/md/src/observe.rs:86-97; histogram and kinetic, observe.wgsl:31-56), 2D
 * engines: a gx x gy density grid over the box, bin (min(u32(coord(x) gx/Lx), gx-1),
 * min(u32(coord(y) gy/Ly), gy-1)) with coord the f32 value of the wrapped position and gx/Lx
 * rounded to f32, stored row-major (by * gx + bx); counts of all particles into `all` and of
 * species `marked` into `marked_counts` (gx * gy words each, either may be NULL), and the
 * half-step kinetic energy of the moving particles into `kinetic` (summed exactly in integers,
 * returned in f64; the reference sums f32). Synchronous. GBMD_E_UNSUPPORTED in 3D. */
int gbmd_observe_grid(gbmd_engine* e, uint32_t gx, uint32_t gy, uint32_t marked, uint32_t* all, uint32_t* marked_counts,
                      double* kinetic);

/* ---- Diagnostics ---- */

/* Verlet-list rebuilds so far and whether any list overflowed (Buffers::read_list_stats). */
int gbmd_list_stats(gbmd_engine* e, uint32_t* rebuilds, int32_t* overflow);
/* FNV-1a hash of the id-ordered state (State::hash, system.rs:460-477; three.rs:280-297). */
int gbmd_state_hash(gbmd_engine* e, uint64_t* hash);
/* Net steps (GpuEngine::steps) and the clock (steps in either direction). */
int gbmd_counters(gbmd_engine* e, int64_t* steps, uint32_t* clock);
/* The energy/impulse ledger (md_core::walls::Ledger, walls.rs:40-50; GpuEngine::read_ledger):
 * GBMD_LEDGER_SLOTS entries each, slot 2 axis + side for walls, GBMD_LEDGER_BATH for the heat
 * bath: the energy given to the system, the normal momentum given to the wall and the hits (the
 * bath's redraws). Each event's f64 energy change and impulse is rounded half away from zero to
 * 2^-24 and summed as an integer, so the totals do not depend on the order of events. */
#define GBMD_LEDGER_SLOTS 7
#define GBMD_LEDGER_BATH 6
int gbmd_read_ledger(gbmd_engine* e, double* energy, double* impulse, uint64_t* hits);
/* GpuEngine::read_compartment_ledger (engine.rs:455-470, walls::CompartmentLedger walls.rs:52-72):
 * the same per slot and per compartment along its wall (compartment c along the other axis of the
 * wall's axis; 0 for the bath and without compartments), slot w, compartment c at [w cap + c] for
 * c < cap (entries past the engine's count are 0). *per_wall receives the engine's count (the
 * most compartments along either axis, 1 without); with all three arrays NULL only that. */
int gbmd_read_compartment_ledger(gbmd_engine* e, uint32_t cap, double* energy, double* impulse, uint64_t* hits, uint32_t* per_wall);
/* The CUDA stream the engine launches on (a cudaStream_t), for event timing by the caller. */
int gbmd_stream(gbmd_engine* e, void** stream);
/* Kernels launched by this engine so far (every launch, graph nodes included). */
int gbmd_launch_count(gbmd_engine* e, uint64_t* launches);

/* Per-phase device timing (the reference's PassTimer, crates/bench/src/main.rs:178-198): run
 * `steps` steps as individual launches with CUDA events around each phase on the engine's
 * stream; returns the mean milliseconds of one force launch and of one list rebuild (all its
 * kernels), and how many rebuilds ran. The state advances by `steps` steps. */
int gbmd_time_phases(gbmd_engine* e, uint32_t steps, double* force_ms, double* rebuild_ms, uint32_t* rebuilds);
/* The same for the persistent step loop of small systems (no counterpart in the reference: its
 * engine has no such loop): at least `steps` steps taken by direct cooperative launches of the
 * loop (each stops at the rebuild trigger or after the engine's block of steps), the list
 * rebuilt between them where the trigger fired. Returns the steps taken, the mean milliseconds
 * per step inside the loop launches and their count; GBMD_E_UNSUPPORTED when the engine does
 * not use the loop. */
int gbmd_time_loop(gbmd_engine* e, uint32_t steps, uint32_t* taken, double* ms_per_step, uint32_t* launches);
/* The velocity-rescale thermostat's kernels (exact kinetic energy, factor, rescale, exact zero
 * momentum) run `reps` times as direct launches with CUDA events around each (a profiler sees
 * them; inside the step graphs it does not): the mean milliseconds. Each run rescales the
 * velocities, as a rescale step does. GBMD_E_INVALID without a thermostat. */
int gbmd_time_thermostat(gbmd_engine* e, uint32_t reps, double* ms);

/* ---- Introspection of the cell binning and the Verlet list (parity tests) ---- */

/* Cell keys, cell starts and the stable sort permutation of the current storage order, exactly
 * as md_ref::CellList::build (crates/md-ref/src/cells.rs:10-32) computes them for `cells` cells
 * per axis (cell_of in f64, cells.rs:53-55; row-major keys). keys[n], start[ncell+1], items[n];
 * `order` (n ids) receives the id of each storage slot the binning saw. */
int gbmd_debug_bin(gbmd_engine* e, const uint32_t* cells, uint32_t* keys, uint32_t* start,
                   uint32_t* items, uint32_t* order);
/* The Verlet list as built now: for each id, its neighbour ids (any order), `counts[id]` of
 * them, packed in id order into `nbr` (capacity `nbr_cap` entries). */
int gbmd_debug_list(gbmd_engine* e, uint32_t* counts, uint32_t* nbr, uint64_t nbr_cap);
/* No counterpart in the reference. The failure path of the persistent step loop's grid barrier,
 * exercised without a GPU fault: a cooperative launch of `blocks` blocks of which block 0 never
 * arrives, so the others' bounded waits run out (a fraction of a second). Returns what the
 * engine then reports: GBMD_E_TIMEOUT with the barrier's message, the engine in its failed state. */
int gbmd_debug_barrier_timeout(gbmd_engine* e, uint32_t blocks);

/* ---- Seeded initial conditions on the device (md_core::init, crates/md-core/src/init.rs) ---- */

/* Init recipes. */
#define GBMD_INIT_FLUID 0       /* init::fluid: square-ish lattice, jitter 0.1, Maxwell (2D) */
#define GBMD_INIT_TRIANGULAR 1  /* triangular lattice + Maxwell (2D; new, see init spec) */
#define GBMD_INIT_FCC 2         /* three::fcc + three::maxwell (3D) */
#define GBMD_INIT_SLAB 3        /* liquid slab (triangular) + jittered-lattice vapour (2D) */

typedef struct gbmd_init {
    uint32_t recipe;    /* GBMD_INIT_* */
    uint32_t n;
    double t;           /* kT of the Maxwell velocities */
    uint64_t seed;
    double jitter;      /* lattice jitter in sigma */
    double rho_liquid;  /* slab: liquid density */
    double rho_vapour;  /* slab: vapour density */
    double slab_frac;   /* slab: fraction of the long (x) axis the liquid fills */
} gbmd_init;

/* Generate the id-ordered initial state on the device (bit-identical to md_core::init) and copy
 * it to the host arrays (any of which may be NULL). */
int gbmd_init_state(const gbmd_system* sys, const gbmd_init* spec, int64_t* pos, int32_t* vel,
                    uint32_t* species);
/* init::maxwell (crates/md-core/src/init.rs:42-57) and three::maxwell for the given id-ordered
 * species (each drawn at kT = t with its own mass), with the exact zero velocity sum, into `vel`
 * (n * dim words), on the device. */
int gbmd_maxwell(const gbmd_system* sys, const uint32_t* species, uint32_t n, double t, uint64_t seed, int32_t* vel);
/* init::fixed_speed (init.rs:61-74), 2D: every particle at speed sqrt(2 t / m) in a direction
 * drawn on (seed, stream 3, id), with the exact zero velocity sum, on the device. */
int gbmd_fixed_speed(const gbmd_system* sys, const uint32_t* species, uint32_t n, double t, uint64_t seed, int32_t* vel);
/* Create an engine whose state is generated on the device by `spec` (no host round trip). */
int gbmd_create_seeded(const gbmd_system* sys, const gbmd_init* spec, const gbmd_options* opts,
                       gbmd_engine** out);

/* ---- Cell binning without device allocation ---- */

/* Largest particle count gbmd_bin_cells_static accepts. */
#define GBMD_BIN_STATIC_MAX_N 262144u

/* No counterpart in the reference. The cell binning of gbmd_debug_bin (row-major f64 cell keys,
 * the stable sort permutation and the cell starts of md_ref::CellList::build) for callers that
 * cannot allocate device memory: a host that gives the library a fixed arena at start-up and
 * allows no later cudaMalloc, or a stream-ordered hot path where cudaMalloc/cudaFree would
 * synchronise the device. All pointers except `sys` and `cells` are DEVICE pointers the caller
 * owns: `pos` holds n id-ordered interleaved int64 positions (n * dim), and the outputs are
 * keys[n], start[ncell + 1] and items[n]. `stream` is a cudaStream_t (NULL: the legacy default
 * stream); the work is enqueued on it and the call returns without waiting.
 * The scratch is one static device array of about 4.3 MB (4 * GBMD_BIN_STATIC_MAX_N words plus
 * the sort's histograms), which every GPU that loads the library holds until the process
 * exits; n above GBMD_BIN_STATIC_MAX_N is rejected with GBMD_E_INVALID, as are a box length
 * that is not positive and a cell count (product of `cells`) of 2^32 - 1 or more, all before any
 * device work. With n = 0 only start[] is written (zeros). The first call on each
 * device looks up that array's device address (cudaGetSymbolAddress, with that device current),
 * so make the first call on a device before any stream capture. Every call shares the one
 * array: calls that overlap on the GPU (other streams, other threads) race and must be
 * serialised by the caller. The array keeps the last call's contents; nothing in it needs to
 * start at zero, since every word a call reads it has written first. */
int gbmd_bin_cells_static(const gbmd_system* sys, const int64_t* pos, uint32_t n, const uint32_t* cells,
                          uint32_t* keys, uint32_t* start, uint32_t* items, void* stream);

/* ---- Batched replicas: many independent periodic systems in one persistent launch ---- */

typedef struct gbmd_batch gbmd_batch;

/* `systems[k]` with its own initial state, concatenated in `pos/vel/species` at `offsets[k]`
 * (offsets[count] = total particles). */
int gbmd_batch_create(const gbmd_system* systems, uint32_t count, const uint32_t* offsets,
                      const int64_t* pos, const int32_t* vel, const uint32_t* species,
                      const gbmd_options* opts, gbmd_batch** out);
int gbmd_batch_step(gbmd_batch* b, uint64_t steps);
int gbmd_batch_sync(gbmd_batch* b);
/* The id-ordered state of system k. */
int gbmd_batch_read_system(gbmd_batch* b, uint32_t k, int64_t* pos, int32_t* vel, uint32_t* species);
/* Set each system's step clock (IntEngine::clock, on which its heat bath draws) to clocks[k]: a
 * system that continues a run elsewhere keeps its clock. Systems start at 0 otherwise. */
int gbmd_batch_set_clocks(gbmd_batch* b, const uint32_t* clocks);
/* The id-ordered states of every system, concatenated at the batch's offsets (one conversion). */
int gbmd_batch_read_all(gbmd_batch* b, int64_t* pos, int32_t* vel, uint32_t* species);
/* A frame of every system at once: gbmd_observe's energies, virial, temperature and pressure per
 * system into frames[count] (`step` is the batch's steps), and, with rdf_bins > 0, each system's
 * RDF counts (unordered pairs, floor(r rdf_bins / rdf_rmax)) into rdf[count * rdf_bins], system by
 * system; the counts equal a plain engine's exactly, the sums agree to rounding (they are added in
 * another order). _begin enqueues the work and copies on the batch's stream and returns at once;
 * _end waits for them. Stepping is refused while a frame is in flight. */
int gbmd_batch_observe_begin(gbmd_batch* b, uint32_t rdf_bins, double rdf_rmax);
int gbmd_batch_observe_end(gbmd_batch* b, gbmd_frame* frames, uint64_t* rdf);
int gbmd_batch_observe(gbmd_batch* b, gbmd_frame* frames, uint64_t* rdf, uint32_t rdf_bins, double rdf_rmax);
int gbmd_batch_stream(gbmd_batch* b, void** stream);
/* Kernel launches of the batch so far (graph nodes included) and its list rebuilds. */
int gbmd_batch_stats(gbmd_batch* b, uint64_t* launches, uint32_t* rebuilds);
/* System k's ledger, as gbmd_read_ledger: its heat bath's slot (each system keeps its own). */
int gbmd_batch_read_ledger(gbmd_batch* b, uint32_t k, double* energy, double* impulse, uint64_t* hits);
/* The batch's Verlet skin in sigma (the one GBMD_FLAG_TUNE_SKIN chose, or the one asked for). */
int gbmd_batch_skin(gbmd_batch* b, double* skin);
/* The batch's force lanes per particle (the autotuner's choice, or the one asked for). */
int gbmd_batch_force_lanes(gbmd_batch* b, uint32_t* lanes);
/* Per-phase device timing of a batch, as gbmd_time_phases: `steps` steps as individual launches
 * with CUDA events around the force launch and the (all-system) list rebuild. */
int gbmd_batch_time_phases(gbmd_batch* b, uint32_t steps, double* force_ms, double* rebuild_ms, uint32_t* rebuilds);
int gbmd_batch_destroy(gbmd_batch* b);

/* FNV-1a hash of an id-ordered state held on the host: State::hash (system.rs:460-477) for
 * dim 2, State3::hash (three.rs:281-297) for dim 3. */
uint64_t gbmd_hash_state(uint32_t dim, const int64_t* pos, const int32_t* vel, const uint32_t* species, uint32_t n);

/* Self-check of the pair arithmetic on `device`: the engine's own correctly rounded reciprocal
 * and division, used by the pair force for separations above sigma / 8, compared bit for bit
 * with CUDA's __frcp_rn / __fdiv_rn over every f32 of the reciprocal's range [2^50, 2^63), every
 * f32 r2 of each pair type's fast range through the whole LJ chain (PairConsts::eval,
 * crates/md-ref/src/real.rs:125-139), and `random_quotients` seeded random quotients; for a single
 * species with sigma = 1, also `random_quotients` random pairs of separations through the 3D force
 * kernel's packed (f32x2) two-pair kicks against two scalar kicks. `checked`
 * receives the number of cases, `mismatched` those that differ (0 when the arithmetic holds). */
int gbmd_check_pair_math(const gbmd_system* sys, uint64_t random_quotients, int32_t device, uint64_t* checked, uint64_t* mismatched);
/* Self-check of the velocity rescale's integer arithmetic (round(v f) as i32 from the exact
 * product, without f64 arithmetic) against the f64 product and rounding, on `count` seeded
 * random (v, f) pairs on `device`: `mismatched` receives the cases that differ (0 when it holds). */
int gbmd_check_rescale(uint64_t count, int32_t device, uint64_t* checked, uint64_t* mismatched);
/* The device's ln, cos and sin (its fdlibm restatement, which the initial velocities, the heat
 * bath and the thermal walls draw with) at n arguments: out[3 i], out[3 i + 1], out[3 i + 2]. */
int gbmd_debug_libm(const double* x, uint32_t n, double* out);

/* ---- Serving: requests admitted against an HBM budget, stepped concurrently, frames streamed ---- */

#define GBMD_SERVE_RDF_BINS 256

/* One simulation request: a periodic system, its seeded initial state, how many steps, a frame
 * of observables every `frame_every` steps (and after the last), with an RDF of `rdf_bins` bins
 * to `rdf_rmax` (0 bins: none), Verlet skin `skin` (<= 0: 0.3). */
typedef struct gbmd_serve_request {
    gbmd_system sys;
    gbmd_init init;
    uint64_t steps;
    uint32_t frame_every;
    uint32_t rdf_bins;
    double rdf_rmax;
    double skin;
} gbmd_serve_request;

/* A frame delivered to the client. `ready_ns` is when the server had it, in ns since the server
 * was created; on the request's last frame `last` is 1 and `state_hash` the FNV-1a hash of its
 * final id-ordered state. */
typedef struct gbmd_serve_frame {
    uint64_t request;
    gbmd_frame frame;
    uint64_t ready_ns;
    uint32_t index;
    uint32_t last;
    uint64_t state_hash;
    uint64_t rdf[GBMD_SERVE_RDF_BINS];
} gbmd_serve_frame;

typedef struct gbmd_serve_stats_t {
    uint32_t pending;
    uint32_t active;
    uint64_t admitted;
    uint64_t completed;
    uint64_t bytes_in_use;
    uint64_t budget;
    uint64_t atom_steps;
    uint64_t lane_requests; /* requests served in a lane (stepped together in a batch) */
    uint64_t lane_repacks;  /* lane batches built: one per interval boundary where members joined or left */
} gbmd_serve_stats_t;

typedef struct gbmd_server gbmd_server;

/* A server on `device` holding at most `max_active` requests (0: 64) within `hbm_budget_bytes`
 * of device memory. Requests are admitted first come, first served as memory and slots free up.
 * Small requests of one dimension are stepped together in a batch (gbmd_serve_set_lanes), the
 * others each on an engine of their own; all of them overlap on the device. */
int gbmd_serve_create(uint64_t hbm_budget_bytes, uint32_t max_active, int32_t device, gbmd_server** out);
int gbmd_serve_submit(gbmd_server* sv, const gbmd_serve_request* req, uint64_t* request_id);
/* Drive the loop once without blocking on the GPU: collect finished frame intervals, enqueue the
 * next ones, admit waiting requests, and copy out up to `cap` frames. */
int gbmd_serve_poll(gbmd_server* sv, gbmd_serve_frame* frames, uint32_t cap, uint32_t* count);
int gbmd_serve_cancel(gbmd_server* sv, uint64_t request_id);
int gbmd_serve_stats(gbmd_server* sv, gbmd_serve_stats_t* stats);
int gbmd_serve_destroy(gbmd_server* sv);
/* Requests of at most `lane_max_n` particles (default 65,536; 0: none) whose frame cadence divides
 * their steps are served in their dimension's lane: stepped together in one batch with the lane's
 * other members, which share its cadence and RDF shape (those of the lane's first member), joining
 * and leaving it at frame boundaries. Set before the first request. */
int gbmd_serve_set_lanes(gbmd_server* sv, uint32_t lane_max_n);
/* Device bytes a request of this size is charged against the budget. */
uint64_t gbmd_serve_estimate_bytes(const gbmd_system* sys, uint32_t n, double skin);

/* ---- Thread-local error message ---- */

const char* gbmd_last_error(void);
/* Library version string. */
const char* gbmd_version(void);

#ifdef __cplusplus
}
#endif

#endif /* GBMD_H */
