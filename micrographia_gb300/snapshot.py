"""The engine's binary snapshot format (gbmd_snapshot / gbmd_restore), read and written on the
host: a 56-byte header ("GBMDSNP1", version, dim, n, step counter, clock, thermostat phase and the
state's FNV-1a hash) followed by the id-ordered positions (i64), velocities (i32) and species
(u32) of md-core's State / State3. Files in this format resume a run bit for bit."""

import ctypes as C
import struct

import numpy as np

from . import _abi

MAGIC = b"GBMDSNP1"
HEADER = struct.Struct("<8sIIIIqIIQQ")  # magic, version, dim, n, 0, steps, clock, 0, phase, hash


def size(dim, n):
    return HEADER.size + n * (dim * 8 + dim * 4 + 4)


def _hash(dim, pos, vel, species):
    n = len(species)
    return _abi.lib().gbmd_hash_state(
        dim,
        np.ascontiguousarray(pos, np.int64).ctypes.data_as(C.POINTER(C.c_int64)),
        np.ascontiguousarray(vel, np.int32).ctypes.data_as(C.POINTER(C.c_int32)),
        np.ascontiguousarray(species, np.uint32).ctypes.data_as(C.POINTER(C.c_uint32)),
        n,
    )


def pack(dim, pos, vel, species, steps=0, clock=0, phase=0):
    """A snapshot of an id-ordered state (pos/vel shaped (n, dim)) and its counters."""
    pos = np.ascontiguousarray(pos, np.int64).reshape(-1)
    vel = np.ascontiguousarray(vel, np.int32).reshape(-1)
    species = np.ascontiguousarray(species, np.uint32).reshape(-1)
    n = len(species)
    head = HEADER.pack(MAGIC, 1, dim, n, 0, steps, clock, 0, phase, _hash(dim, pos, vel, species))
    return head + pos.tobytes() + vel.tobytes() + species.tobytes()


def unpack(buf):
    """(dim, pos (n, dim), vel (n, dim), species, steps, clock, phase); raises ValueError on a
    malformed or corrupted snapshot (the arrays must match the stored hash)."""
    if len(buf) < HEADER.size:
        raise ValueError("not a snapshot (too short)")
    magic, ver, dim, n, _, steps, clock, _, phase, h = HEADER.unpack_from(buf, 0)
    if magic != MAGIC or ver != 1:
        raise ValueError("not a snapshot (magic or version)")
    if len(buf) != size(dim, n):
        raise ValueError("snapshot size does not match its header")
    o = HEADER.size
    pos = np.frombuffer(buf, np.int64, n * dim, o).reshape(n, dim)
    o += n * dim * 8
    vel = np.frombuffer(buf, np.int32, n * dim, o).reshape(n, dim)
    o += n * dim * 4
    species = np.frombuffer(buf, np.uint32, n, o)
    if _hash(dim, pos, vel, species) != h:
        raise ValueError("snapshot corrupted (state hash mismatch)")
    return dim, pos, vel, species, steps, clock, phase
