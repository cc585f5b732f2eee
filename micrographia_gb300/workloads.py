"""The benchmark workloads, as seeded synthetic systems (no dataset is
involved): each function returns systems and device-init recipes, never particle data.

- config2: 3D LJ liquid, FCC N = 1,048,576 at rho 0.8442, T 0.72 (the LAMMPS in.lj shape).
- config3: 2D liquid-vapour slab, N = 2^24 in a 4:1 box, liquid rho 0.70 over the central
  quarter, vapour 0.05, rescale to T = 0.45 every 10 steps.
- config4: 1024 independent 2D LJ systems, N = floor(256 * 256^u) (log-uniform in [256, 65536]),
  rho ~ U[0.3, 0.8], T ~ U[0.5, 1.5], seed base + k; u, rho and T drawn from Threefry streams 10,
  11 and 12 of the base seed.
- config5: a Poisson stream of 2D/3D requests with N log-uniform in [1024, 2^20].
"""

import math

from . import _abi
from .core import Pair, System, System3, box_for, cube_for
from .engine import make_init

MASK = 0xFFFFFFFF


def threefry2x32(c0, c1, k0, k1):
    """Threefry-2x32-20 (Random123), as gpu-prims/src/threefry.rs:7-22."""
    rot = (13, 15, 26, 6, 17, 29, 16, 24)
    ks = (k0, k1, 0x1BD11BDA ^ k0 ^ k1)
    x0, x1 = (c0 + k0) & MASK, (c1 + k1) & MASK
    for r in range(20):
        x0 = (x0 + x1) & MASK
        s = rot[r % 8]
        x1 = ((x1 << s) | (x1 >> (32 - s))) & MASK
        x1 ^= x0
        if r & 3 == 3:
            i = (r >> 2) + 1
            x0 = (x0 + ks[i % 3]) & MASK
            x1 = (x1 + ks[(i + 1) % 3] + i) & MASK
    return x0, x1


def uniform(seed, stream, i):
    """threefry::uniform (threefry.rs:35-37): 53 random bits in [0, 1)."""
    a, b = threefry2x32(i & MASK, stream, seed & MASK, (seed >> 32) & MASK)
    bits = ((a << 21) ^ (b >> 11)) & ((1 << 53) - 1)
    return bits * (1.0 / (1 << 53))


def config2(n=1 << 20):
    sys3 = System3(cube_for(n, 0.8442), 0.005, Pair.lj(2.5), [1.0])
    return sys3, make_init(_abi.INIT_FCC, n, 0.72, 1, 0.05)


def config3(n=1 << 24):
    area = n / (0.25 * 0.70 + 0.75 * 0.05)
    sys_ = System(box_for(n, n / area, 4.0), 0.005, Pair.lj(2.5), [1.0])
    return sys_, make_init(_abi.INIT_SLAB, n, 0.45, 1, 0.1, 0.70, 0.05, 0.25)


def config4(count=1024, base_seed=1, n_min=256, n_max=65536):
    out = []
    ratio = n_max / n_min
    for k in range(count):
        u = uniform(base_seed, 10, k)
        n = int(math.floor(n_min * ratio**u))
        rho = 0.3 + 0.5 * uniform(base_seed, 11, k)
        t = 0.5 + uniform(base_seed, 12, k)
        seed = base_seed + k
        sys_ = System(box_for(n, rho, 1.0), 0.005, Pair.lj(2.5), [1.0]).with_seed(seed)
        out.append((sys_, make_init(_abi.INIT_FLUID, n, t, seed, 0.1)))
    return out


def config5(count, rate, base_seed=1, n_min=1024, n_max=1 << 20):
    """Poisson arrivals at `rate` requests per second: (arrival time s, system, init) each."""
    out = []
    t = 0.0
    for k in range(count):
        t += -math.log(1.0 - uniform(base_seed, 20, k)) / rate
        u = uniform(base_seed, 21, k)
        n = int(math.floor(n_min * (n_max / n_min) ** u))
        rho = 0.3 + 0.55 * uniform(base_seed, 22, k)
        temp = 0.5 + uniform(base_seed, 23, k)
        seed = base_seed + 1000 + k
        if uniform(base_seed, 24, k) < 0.5:
            sys_ = System(box_for(n, rho, 1.0), 0.005, Pair.lj(2.5), [1.0]).with_seed(seed)
            init = make_init(_abi.INIT_FLUID, n, temp, seed, 0.1)
        else:
            sys_ = System3(cube_for(n, rho), 0.005, Pair.lj(2.5), [1.0]).with_seed(seed)
            init = make_init(_abi.INIT_FCC, n, temp, seed, 0.05)
        out.append((t, sys_, init))
    return out


def _profile_run(name):
    """Runs one small workload on cuda:0 so that a profiler can capture the kernels it exercises
    (each run ends by itself within seconds):
    - frames3d: the 3D liquid (FCC N = 2^20, rho 0.8442, T 0.72, skin 0.3), 20 steps, then three
      frames (the energy/virial pass k_kicks<3> and a 200-bin RDF to r = 5, k_rdf<3>);
    - loop3d: one 3D liquid of N = 32,000 stepped 512 times by the persistent step loop, then 512
      more by direct launches of the loop (k_force_loop; a profiler cannot see kernels inside the
      graphs' conditional nodes);
    - batch: the first 256 of the 1024 batched 2D replicas, 300 steps in 100-step graphs, then 50
      steps by direct launches (k_bforce_list, k_bbuild_list), then two frames of every system
      (k_bframe, and a 200-bin RDF to r = 5, k_brdf);
    - scenario2d: a 2D Kremer-Grest melt of 32,768 chains of 32 beads (N = 2^20, rho 0.3, WCA
      beads, FENE bonds) between a soft floor and a hard roof, under a piston driven down at
      0.1 sigma/tau from the roof; 50 steps in graphs, then 30 by direct launches (the force
      kernel with its scenario epilogue, k_piston_tick, and k_slot_of with each list build);
    - thermo2d: the liquid-vapour slab of configs[2] at a quarter of its size (N = 2^22) with its
      velocity rescale to T = 0.45 every 10 steps, 20 steps, then the thermostat's kernels four
      times by direct launches (k_ke_exact, k_thermo_factor, k_rescale, k_zero_apply);
    - half3d: the 3D liquid of configs[1] on the opt-in half-shell lists, 20 steps in graphs,
      then 20 by direct launches (k_build_half, k_force_half, k_leap_half);
    - slab2d: the liquid-vapour slab of configs[2] at a quarter of its size (N = 2^22), skin 0.4,
      100 steps in graphs, then 30 by direct launches (k_force_list<2>, k_build_list<2> and the
      binning)."""
    from .engine import BatchEngine, ForceMode, GpuEngine3, init_state

    if name == "frames3d":
        sys3, spec = config2()
        with GpuEngine3(sys3, None, ForceMode.verlet_with_skin(sys3, spec.n, 0.3), init=spec) as e:
            e.step(20)
            for _ in range(3):
                f, _, _ = e.observe(rdf_bins=200, rdf_rmax=5.0)
            print(f"frames3d: T {f.temperature:.4f} P {f.pressure:.4f}")
    elif name == "loop3d":
        n = 32_000
        sys3 = System3(cube_for(n, 0.8442), 0.005, Pair.lj(2.5), [1.0])
        spec = make_init(_abi.INIT_FCC, n, 0.72, 1, 0.05)
        with GpuEngine3(sys3, None, ForceMode.verlet_with_skin(sys3, n, 0.3), init=spec) as e:
            e.step(512)
            taken, ms, launches = e.time_loop(512)
            print(f"loop3d: {taken} steps in {launches} loop launches, {ms * 1e3:.1f} us per step; rebuilds {e.read_list_stats()[0]}")
    elif name == "batch":
        cfg = config4()[:256]
        systems = [s for s, _ in cfg]
        states = [init_state(s, sp.recipe, sp.n, sp.t, sp.seed, sp.jitter) for s, sp in cfg]
        with BatchEngine(systems, states, ForceMode.verlet_with_skin(None, 0, 0.6), block_steps=100) as b:
            b.step(300)
            b.wait()
            f, r, nr = b.time_phases(50)
            print(f"batch: {sum(st.n() for st in states)} particles, force {f:.3f} ms, rebuild {r:.3f} ms ({nr} in 50 steps)")
            for _ in range(2):
                frames, rdf = b.observe(rdf_bins=200, rdf_rmax=5.0)
            print(f"batch frames: T[0] {frames[0].temperature:.4f}, RDF counts {int(rdf.sum())}")
    elif name == "scenario2d":
        import numpy as np

        from .core import Bond, Piston, State, Wall, chains, to_f64
        from .engine import GpuEngine

        n_chains, length = 32768, 32
        n = n_chains * length
        sys2 = System(box_for(n, 0.3, 1.0), 0.005, Pair.wca(), [1.0]).with_walls(1, Wall.soft(), Wall.hard())
        pos, bonds = chains(sys2, n_chains, length, 0.97)
        sys2.with_bonds([Bond.kremer_grest()], bonds)
        sys2.with_piston(Piston.speed_drive(-0.1), to_f64(sys2.box_len[1]), 2.0)
        vel = init_state(sys2, _abi.INIT_FLUID, n, 1.0, 5).vel  # Maxwell velocities with zero sum
        st = State(pos, vel, np.zeros(n, np.uint32))
        with GpuEngine(sys2, st, ForceMode.verlet_with_skin(sys2, n, 0.3)) as e:
            e.step(50)
            f, r, nr = e.time_phases(30)
            w, v, work = e.piston()
            print(f"scenario2d: N {n}, force pass {f:.3f} ms, rebuild {r:.3f} ms ({nr} in 30 steps), piston at {to_f64(w):.2f}")
    elif name == "thermo2d":
        from .engine import GpuEngine

        sys2, spec = config3(1 << 22)
        with GpuEngine(sys2, None, ForceMode.verlet_with_skin(sys2, spec.n, 0.4), init=spec, rescale_every=10, rescale_t=0.45) as e:
            e.step(20)
            ms = e.time_thermostat(4)
            print(f"thermo2d: N {spec.n}, thermostat {ms:.3f} ms")
    elif name == "slab2d":
        from .engine import GpuEngine

        sys2, spec = config3(1 << 22)
        with GpuEngine(sys2, None, ForceMode.verlet_with_skin(sys2, spec.n, 0.4), init=spec, rescale_every=10, rescale_t=0.45) as e:
            e.step(100)
            f, r, nr = e.time_phases(30)
            print(f"slab2d: N {spec.n}, force {f:.3f} ms, rebuild {r:.3f} ms ({nr} in 30 steps)")
    elif name == "half3d":
        sys3, spec = config2()
        with GpuEngine3(sys3, None, ForceMode.verlet_with_skin(sys3, spec.n, 0.3), init=spec, flags=_abi.FLAG_HALF_LISTS) as e:
            e.step(20)
            f, r, nr = e.time_phases(20)
            print(f"half3d: force {f:.3f} ms, rebuild {r:.3f} ms ({nr} in 20 steps)")
    else:
        raise SystemExit(f"unknown workload {name!r}: frames3d, loop3d, batch, scenario2d, thermo2d, half3d or slab2d")


if __name__ == "__main__":
    import sys

    _profile_run(sys.argv[1] if len(sys.argv) > 1 else "")
