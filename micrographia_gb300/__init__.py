"""micrographia_gb300 — a GB300-native integer fixed-point Lennard-Jones MD engine.

The Python face of the engine mirrors the interface micrographia's scenarios and tests drive:
md-core's `Pair`, `System`, `State`, `System3`, `State3`, `Thermostat` (the Andersen bath, with
the `with_thermostat` / `with_fan` / `with_bath_layer` builders) and `init` helpers
(crates/md-core/src/{pair,system,init,three}.rs), and the engines `GpuEngine` / `GpuEngine3`
(crates/md/src/engine.rs:598-1098, engine3.rs:334-648) with `step`, `reverse`, `kicks`,
`read_state`, `upload`, `energy`, `flip_bit`, `read_list_stats`, `read_ledger` and `ForceMode`;
the Observer's `Reading` with `mixing` and `segregation` (crates/md/src/observe.rs);
`BatchEngine` and `Server` run many systems at once.

All compute runs in the CUDA library libgbmd.so through its C ABI (include/gbmd.h); importing
works without a GPU, and every engine call fails loudly when the library or the GPU is missing.
"""

from .core import (
    DT,
    ONE,
    Bond,
    ForceMode,
    Pair,
    Piston,
    State,
    State3,
    System,
    System3,
    Thermostat,
    Wall,
    box_for,
    chains,
    cube_for,
    fcc_cells,
    to_f64,
    to_fixed,
)
from .engine import BatchEngine, GpuEngine, GpuEngine3, Server, init_state
from .observe import Reading, mixing, segregation
from . import checks, init, workloads

__all__ = [
    "DT",
    "ONE",
    "Bond",
    "ForceMode",
    "Pair",
    "Piston",
    "State",
    "State3",
    "System",
    "System3",
    "Thermostat",
    "Wall",
    "GpuEngine",
    "GpuEngine3",
    "BatchEngine",
    "Server",
    "Reading",
    "mixing",
    "segregation",
    "box_for",
    "chains",
    "cube_for",
    "fcc_cells",
    "to_f64",
    "to_fixed",
    "checks",
    "init",
    "init_state",
    "workloads",
]
