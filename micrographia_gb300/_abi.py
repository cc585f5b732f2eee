"""ctypes mirror of include/gbmd.h and the loader of the engine library.

The engine is the C-ABI shared library micrographia_gb300/_build/libgbmd.so, built in-tree by
micrographia_gb300/build.py. Loading fails loudly when it is missing: there is no CPU fallback.
"""

import ctypes as C
import os

MAX_SPECIES = 4

OK = 0
E_INVALID = -1
E_NOMEM = -2
E_BUDGET = -3
E_OVERFLOW = -4
E_NONFINITE = -5
E_TIMEOUT = -6
E_CUDA = -7
E_UNSUPPORTED = -8
E_NOTFOUND = -9

MODE_AUTO = 0
MODE_CELLS = 1
MODE_VERLET = 2
ARITH_F32 = 0
ARITH_INT = 1

INIT_FLUID = 0
INIT_TRIANGULAR = 1
INIT_FCC = 2
INIT_SLAB = 3

BIN_STATIC_MAX_N = 262144  # GBMD_BIN_STATIC_MAX_N


class gbmd_pair(C.Structure):
    _fields_ = [("eps", C.c_double), ("sigma", C.c_double), ("rc", C.c_double)]


class gbmd_system(C.Structure):
    _fields_ = [
        ("dim", C.c_uint32),
        ("nspecies", C.c_uint32),
        ("box_len", C.c_int64 * 3),
        ("dt", C.c_double),
        ("masses", C.c_double * MAX_SPECIES),
        ("pairs", gbmd_pair * (MAX_SPECIES * MAX_SPECIES)),
        ("gravity", C.c_double * 3),
        ("seed", C.c_uint64),
        ("periodic", C.c_uint32),
        ("pinned", C.c_uint32),
        ("bath", C.c_uint32),
        ("bath_species", C.c_uint32),
        ("bath_axis", C.c_uint32),
        ("_bath_pad", C.c_uint32),
        ("bath_t", C.c_double),
        ("bath_rate", C.c_double),
        ("bath_drift", C.c_double),
        ("bath_region", C.c_int64 * 2),
        ("wall_kind", (C.c_uint32 * 2) * 3),
        ("wall_t", (C.c_double * 2) * 3),
        ("membrane", C.c_uint32),
        ("membrane_axis", C.c_uint32),
        ("membrane_blocks", C.c_uint32),
        ("membrane_pore_shift", C.c_uint32),
        ("membrane_position", C.c_int64),
        ("membrane_pore_width", C.c_int64),
        ("compartments", C.c_uint32 * 2),
        ("compartments_diathermal", C.c_uint32),
        ("_compartments_pad", C.c_uint32),
    ]


MAX_BONDS = 4  # system.rs:66, bonds per particle
MAX_BOND_TYPES = 4  # system.rs:67
BOND_HARMONIC = 0  # md_core::BondType::Harmonic
BOND_FENE = 1  # md_core::BondType::Fene


class gbmd_bond_type(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("_pad", C.c_uint32), ("k", C.c_double), ("r0", C.c_double)]


PISTON_NONE = 0
PISTON_SPEED = 1  # md_core::PistonDrive::Speed
PISTON_FREE = 2  # PistonDrive::Free


class gbmd_piston(C.Structure):
    _fields_ = [
        ("drive", C.c_uint32),
        ("_pad", C.c_uint32),
        ("speed", C.c_double),
        ("mass", C.c_double),
        ("force", C.c_double),
        ("start", C.c_double),
        ("min", C.c_double),
    ]


WALL_HARD = 1  # md_core::Wall::Hard: exact mirror
WALL_SOFT = 2  # Wall::Soft: WCA repulsion from the wall
WALL_THERMAL = 3  # Wall::Thermal(t): a hit draws a Maxwell-flux velocity at kT = t


LEDGER_SLOTS = 7  # md_core::walls::WALLS: 2 axis + side, membrane faces 4 and 5, the bath
LEDGER_BATH = 6


FLAG_WHOLE_CELLS = 1  # list builds scan whole neighbour cells (no slab sub-buckets)
FLAG_NO_STEP_LOOP = 2  # small systems step through per-step graph nodes, not the persistent loop
FLAG_TUNE_SKIN = 4  # batches: time each skin of 0.3..0.7 sigma on the given state, keep the fastest
FLAG_HALF_LISTS = 1 << 14  # half-shell lists (3D, one species): each pair evaluated once; full lists by default
FLAG_NO_PATH_BOUND = 1 << 15  # 2D: always run the displacement test (no path bound): comparisons


def build_lanes_flag(lanes):
    """gbmd_options.flags bits 4-7: lanes per particle of the list build (0 chooses by size)."""
    if lanes not in (0, 1, 2, 4, 8):
        raise ValueError("build lanes must be 0, 1, 2, 4 or 8")
    return lanes << 4


def force_lanes_flag(lanes):
    """gbmd_options.flags bits 8-12: lanes per particle of the force step (0 chooses by size)."""
    if lanes not in (0, 1, 2, 4, 8, 16):
        raise ValueError("force lanes must be 0, 1, 2, 4, 8 or 16")
    return lanes << 8


class gbmd_options(C.Structure):
    _fields_ = [
        ("mode", C.c_int32),
        ("arith", C.c_int32),
        ("skin", C.c_double),
        ("cap", C.c_uint32),
        ("block_steps", C.c_uint32),
        ("device", C.c_int32),
        ("threads", C.c_uint32),
        ("rescale_every", C.c_uint32),
        ("flags", C.c_uint32),
        ("rescale_t", C.c_double),
    ]


class gbmd_frame(C.Structure):
    _fields_ = [
        ("step", C.c_uint64),
        ("kinetic", C.c_double),
        ("potential", C.c_double),
        ("virial", C.c_double),
        ("temperature", C.c_double),
        ("pressure", C.c_double),
        ("volume", C.c_double),
        ("n", C.c_uint32),
        ("dim", C.c_uint32),
    ]


class gbmd_init(C.Structure):
    _fields_ = [
        ("recipe", C.c_uint32),
        ("n", C.c_uint32),
        ("t", C.c_double),
        ("seed", C.c_uint64),
        ("jitter", C.c_double),
        ("rho_liquid", C.c_double),
        ("rho_vapour", C.c_double),
        ("slab_frac", C.c_double),
    ]


class gbmd_serve_request(C.Structure):
    _fields_ = [
        ("sys", gbmd_system),
        ("init", gbmd_init),
        ("steps", C.c_uint64),
        ("frame_every", C.c_uint32),
        ("rdf_bins", C.c_uint32),
        ("rdf_rmax", C.c_double),
        ("skin", C.c_double),
    ]


SERVE_RDF_BINS = 256


class gbmd_serve_frame(C.Structure):
    _fields_ = [
        ("request", C.c_uint64),
        ("frame", gbmd_frame),
        ("ready_ns", C.c_uint64),
        ("index", C.c_uint32),
        ("last", C.c_uint32),
        ("state_hash", C.c_uint64),
        ("rdf", C.c_uint64 * SERVE_RDF_BINS),
    ]


class gbmd_serve_stats_t(C.Structure):
    _fields_ = [
        ("pending", C.c_uint32),
        ("active", C.c_uint32),
        ("admitted", C.c_uint64),
        ("completed", C.c_uint64),
        ("bytes_in_use", C.c_uint64),
        ("budget", C.c_uint64),
        ("atom_steps", C.c_uint64),
        ("lane_requests", C.c_uint64),
        ("lane_repacks", C.c_uint64),
    ]


P = C.POINTER
VP = C.c_void_p
_I64P = P(C.c_int64)
_I32P = P(C.c_int32)
_U32P = P(C.c_uint32)
_U64P = P(C.c_uint64)
_DP = P(C.c_double)

# (name, restype, argtypes): every entry point declared in include/gbmd.h.
SIGNATURES = [
    ("gbmd_create", C.c_int, [P(gbmd_system), _I64P, _I32P, _U32P, C.c_uint32, P(gbmd_options), P(VP)]),
    ("gbmd_destroy", C.c_int, [VP]),
    ("gbmd_step", C.c_int, [VP, C.c_uint64]),
    ("gbmd_sync", C.c_int, [VP]),
    ("gbmd_reverse", C.c_int, [VP]),
    ("gbmd_read_state", C.c_int, [VP, _I64P, _I32P, _U32P]),
    ("gbmd_upload", C.c_int, [VP, _I64P, _I32P, _U32P]),
    ("gbmd_kicks", C.c_int, [VP, _I32P, _DP]),
    ("gbmd_kicks_f64", C.c_int, [VP, _I32P, _DP]),
    ("gbmd_snapshot_bytes", C.c_size_t, [C.c_uint32, C.c_uint32]),
    ("gbmd_snapshot", C.c_int, [VP, VP, C.c_size_t, P(C.c_size_t)]),
    ("gbmd_restore", C.c_int, [VP, VP, C.c_size_t]),
    ("gbmd_flip_bit", C.c_int, [VP, C.c_uint32, C.c_uint32, C.c_uint32]),
    ("gbmd_kick_region", C.c_int, [VP, _DP, _DP, C.c_double, _DP]),
    ("gbmd_set_species", C.c_int, [VP, _U32P, C.c_uint32, C.c_uint32]),
    ("gbmd_set_species_velocity", C.c_int, [VP, C.c_uint32, _DP]),
    ("gbmd_sort_now", C.c_int, [VP]),
    ("gbmd_update_system", C.c_int, [VP, P(gbmd_system)]),
    ("gbmd_set_bonds", C.c_int, [VP, P(gbmd_bond_type), C.c_uint32, P(C.c_uint32), C.c_uint32]),
    ("gbmd_set_piston", C.c_int, [VP, P(gbmd_piston)]),
    ("gbmd_read_piston", C.c_int, [VP, P(C.c_int64), P(C.c_int32), P(C.c_double), P(C.c_double)]),
    ("gbmd_set_piston_speed", C.c_int, [VP, C.c_double]),
    ("gbmd_read_kinetic", C.c_int, [VP, P(C.c_double), P(C.c_uint32), P(C.c_double)]),
    ("gbmd_maxwell", C.c_int, [P(gbmd_system), P(C.c_uint32), C.c_uint32, C.c_double, C.c_uint64, P(C.c_int32)]),
    ("gbmd_fixed_speed", C.c_int, [P(gbmd_system), P(C.c_uint32), C.c_uint32, C.c_double, C.c_uint64, P(C.c_int32)]),
    ("gbmd_observe_grid", C.c_int, [VP, C.c_uint32, C.c_uint32, C.c_uint32, P(C.c_uint32), P(C.c_uint32), P(C.c_double)]),
    ("gbmd_read_compartment_ledger", C.c_int, [VP, C.c_uint32, P(C.c_double), P(C.c_double), P(C.c_uint64), P(C.c_uint32)]),
    ("gbmd_add_bond", C.c_int, [VP, C.c_uint32, C.c_uint32, C.c_uint32, P(C.c_int32)]),
    ("gbmd_remove_bond", C.c_int, [VP, C.c_uint32, C.c_uint32, P(C.c_int32)]),
    ("gbmd_flip_species_bit", C.c_int, [VP, C.c_uint32, C.c_uint32, C.c_uint32]),
    ("gbmd_energy", C.c_int, [VP, _DP, _DP]),
    ("gbmd_observe", C.c_int, [VP, P(gbmd_frame), _U64P, C.c_uint32, C.c_double, _U64P, C.c_uint32, C.c_uint32]),
    ("gbmd_observe_begin", C.c_int, [VP, C.c_uint32, C.c_double, C.c_uint32, C.c_uint32]),
    ("gbmd_observe_end", C.c_int, [VP, P(gbmd_frame), _U64P, _U64P]),
    ("gbmd_list_stats", C.c_int, [VP, _U32P, _I32P]),
    ("gbmd_state_hash", C.c_int, [VP, _U64P]),
    ("gbmd_counters", C.c_int, [VP, _I64P, _U32P]),
    ("gbmd_stream", C.c_int, [VP, P(VP)]),
    ("gbmd_launch_count", C.c_int, [VP, _U64P]),
    ("gbmd_time_phases", C.c_int, [VP, C.c_uint32, _DP, _DP, _U32P]),
    ("gbmd_time_loop", C.c_int, [VP, C.c_uint32, _U32P, _DP, _U32P]),
    ("gbmd_debug_bin", C.c_int, [VP, _U32P, _U32P, _U32P, _U32P, _U32P]),
    ("gbmd_debug_list", C.c_int, [VP, _U32P, _U32P, C.c_uint64]),
    ("gbmd_debug_barrier_timeout", C.c_int, [VP, C.c_uint32]),
    ("gbmd_init_state", C.c_int, [P(gbmd_system), P(gbmd_init), _I64P, _I32P, _U32P]),
    ("gbmd_create_seeded", C.c_int, [P(gbmd_system), P(gbmd_init), P(gbmd_options), P(VP)]),
    ("gbmd_bin_cells_static", C.c_int, [P(gbmd_system), C.c_void_p, C.c_uint32, _U32P, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("gbmd_batch_create", C.c_int, [P(gbmd_system), C.c_uint32, _U32P, _I64P, _I32P, _U32P, P(gbmd_options), P(VP)]),
    ("gbmd_batch_step", C.c_int, [VP, C.c_uint64]),
    ("gbmd_batch_sync", C.c_int, [VP]),
    ("gbmd_batch_read_system", C.c_int, [VP, C.c_uint32, _I64P, _I32P, _U32P]),
    ("gbmd_batch_read_all", C.c_int, [VP, _I64P, _I32P, _U32P]),
    ("gbmd_batch_force_lanes", C.c_int, [VP, _U32P]),
    ("gbmd_batch_set_clocks", C.c_int, [VP, _U32P]),
    ("gbmd_batch_observe_begin", C.c_int, [VP, C.c_uint32, C.c_double]),
    ("gbmd_batch_observe_end", C.c_int, [VP, P(gbmd_frame), P(C.c_uint64)]),
    ("gbmd_batch_observe", C.c_int, [VP, P(gbmd_frame), P(C.c_uint64), C.c_uint32, C.c_double]),
    ("gbmd_batch_stream", C.c_int, [VP, P(VP)]),
    ("gbmd_batch_stats", C.c_int, [VP, _U64P, _U32P]),
    ("gbmd_batch_skin", C.c_int, [VP, C.POINTER(C.c_double)]),
    ("gbmd_batch_time_phases", C.c_int, [VP, C.c_uint32, _DP, _DP, _U32P]),
    ("gbmd_batch_read_ledger", C.c_int, [VP, C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_double), _U64P]),
    ("gbmd_read_ledger", C.c_int, [VP, C.POINTER(C.c_double), C.POINTER(C.c_double), _U64P]),
    ("gbmd_batch_destroy", C.c_int, [VP]),
    ("gbmd_serve_create", C.c_int, [C.c_uint64, C.c_uint32, C.c_int32, P(VP)]),
    ("gbmd_serve_submit", C.c_int, [VP, P(gbmd_serve_request), _U64P]),
    ("gbmd_serve_poll", C.c_int, [VP, P(gbmd_serve_frame), C.c_uint32, _U32P]),
    ("gbmd_serve_cancel", C.c_int, [VP, C.c_uint64]),
    ("gbmd_serve_stats", C.c_int, [VP, P(gbmd_serve_stats_t)]),
    ("gbmd_serve_destroy", C.c_int, [VP]),
    ("gbmd_serve_estimate_bytes", C.c_uint64, [P(gbmd_system), C.c_uint32, C.c_double]),
    ("gbmd_serve_set_lanes", C.c_int, [VP, C.c_uint32]),
    ("gbmd_debug_libm", C.c_int, [P(C.c_double), C.c_uint32, P(C.c_double)]),
    ("gbmd_time_thermostat", C.c_int, [VP, C.c_uint32, P(C.c_double)]),
    ("gbmd_check_rescale", C.c_int, [C.c_uint64, C.c_int32, _U64P, _U64P]),
    ("gbmd_hash_state", C.c_uint64, [C.c_uint32, _I64P, _I32P, _U32P, C.c_uint32]),
    ("gbmd_check_pair_math", C.c_int, [P(gbmd_system), C.c_uint64, C.c_int32, P(C.c_uint64), P(C.c_uint64)]),
    ("gbmd_last_error", C.c_char_p, []),
    ("gbmd_version", C.c_char_p, []),
]

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgbmd.so")
HEADER_PATH = os.path.join(HERE, "..", "include", "gbmd.h")

_lib = None


class GbmdError(RuntimeError):
    """A failed engine call: the status code and the library's message."""

    def __init__(self, code, message):
        super().__init__(f"gbmd error {code}: {message}")
        self.code = code


def lib():
    """Load libgbmd.so (once). Raises if the CUDA extension has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"the CUDA engine library {LIB_PATH} is missing: run micrographia_gb300.build.build() "
                "(there is no CPU fallback)"
            )
        l = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def check(code):
    if code != OK:
        msg = lib().gbmd_last_error()
        raise GbmdError(code, msg.decode() if msg else "")
    return code
