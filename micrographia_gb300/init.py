"""Seeded initial conditions, generated on the device (gbmd_init_state, gbmd_maxwell): the mirror
of md-core's init.rs (fluid: lattice + maxwell, 1 sigma clear of any walls; maxwell for given
species) and three.rs (fcc + maxwell), plus this engine's triangular lattice and liquid-vapour
slab. Bit-identical to the CPU definitions."""

import ctypes as C

import numpy as np

from . import _abi
from .core import DT, System, System3, box_for, cube_for  # noqa: F401
from .engine import init_state

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
