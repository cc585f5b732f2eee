"""Seeded initial conditions, generated on the device (gbmd_init_state): the mirror of
md-core's init.rs (fluid: lattice + maxwell) and three.rs (fcc + maxwell), plus this engine's
triangular lattice and liquid-vapour slab. Bit-identical to the CPU definitions."""

from . import _abi
from .core import DT, System, System3, box_for, cube_for  # noqa: F401
from .engine import init_state

STREAM_VELOCITY = 1
STREAM_JITTER = 2
STREAM_DIRECTION = 3


def fluid(sys: System, n, t, seed):
    """init::fluid (init.rs:107-121) on a periodic box: lattice with jitter 0.1 + Maxwell at t."""
    return init_state(sys, _abi.INIT_FLUID, n, t, seed, jitter=0.1)


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
