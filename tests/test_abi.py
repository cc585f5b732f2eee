"""The C-ABI library: it loads without a GPU and exports every entry point include/gbmd.h
declares (no compute calls: those need a device)."""

import ctypes as C
import re

import numpy as np
import pytest

from micrographia_gb300 import _abi


def header_functions():
    text = open(_abi.HEADER_PATH).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbmd_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = header_functions()
    for must in ["gbmd_create", "gbmd_step", "gbmd_sync", "gbmd_reverse", "gbmd_read_state", "gbmd_upload", "gbmd_kicks",
                 "gbmd_energy", "gbmd_observe", "gbmd_list_stats", "gbmd_state_hash", "gbmd_destroy", "gbmd_last_error"]:
        assert must in names


def test_library_exports_every_declared_symbol(engine_lib):
    for name in header_functions():
        assert hasattr(engine_lib, name), name


def test_python_signatures_cover_the_header():
    declared = set(header_functions())
    bound = {name for name, _, _ in _abi.SIGNATURES}
    assert declared == bound, (declared - bound, bound - declared)


def test_struct_layouts_match_the_header():
    # sizes follow from the header's field order on LP64 (no packing pragmas)
    assert C.sizeof(_abi.gbmd_pair) == 24
    # ... + the heat bath: four u32 (bath, species, axis, pad), t, rate, drift, region[2];
    # + the walls: wall_kind[3][2] (u32), wall_t[3][2] (f64); + the membrane: four u32, two i64;
    # + the compartments: four u32
    assert C.sizeof(_abi.gbmd_system) == 4 + 4 + 24 + 8 + 32 + 16 * 24 + 24 + 8 + 4 + 4 + 16 + 24 + 16 + 24 + 48 + 16 + 16 + 16
    assert C.sizeof(_abi.gbmd_options) == 48
    assert C.sizeof(_abi.gbmd_frame) == 64


def test_host_hash_matches_the_oracle(engine_lib, O):
    import numpy as np

    from micrographia_gb300 import Pair, System, System3, box_for, cube_for

    sys_ = System(box_for(300, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0])
    s = O.fluid(sys_, 300, 1.0, 3)
    h = O.lib().oracle_state_hash(2, s.pos.ctypes.data_as(C.POINTER(C.c_int64)), s.vel.ctypes.data_as(C.POINTER(C.c_int32)),
                                  s.species.ctypes.data_as(C.POINTER(C.c_uint32)), s.n())
    assert s.hash() == h
    sys3 = System3(cube_for(256, 0.8), 0.005, Pair.lj(2.5), [1.0])
    s3 = O.fcc_maxwell(sys3, 256, 1.0, 3)
    h3 = O.lib().oracle_state_hash(3, s3.pos.ctypes.data_as(C.POINTER(C.c_int64)), s3.vel.ctypes.data_as(C.POINTER(C.c_int32)),
                                   s3.species.ctypes.data_as(C.POINTER(C.c_uint32)), s3.n())
    assert s3.hash() == h3


def test_snapshot_format_round_trip_and_corruption():
    """The snapshot format on the host: pack / unpack round trip, the size rule, and a flipped
    bit anywhere in the arrays rejected through the stored state hash."""
    from micrographia_gb300 import snapshot

    rng = np.random.default_rng(4)
    for dim, n in ((2, 37), (3, 64)):
        pos = rng.integers(-(1 << 40), 1 << 40, (n, dim))
        vel = rng.integers(-(1 << 30), 1 << 30, (n, dim)).astype(np.int32)
        sp = rng.integers(0, 4, n).astype(np.uint32)
        buf = snapshot.pack(dim, pos, vel, sp, steps=1234, clock=77, phase=9)
        assert len(buf) == snapshot.size(dim, n)
        d2, p2, v2, s2, steps, clock, phase = snapshot.unpack(buf)
        assert (d2, steps, clock, phase) == (dim, 1234, 77, 9)
        assert np.array_equal(p2, pos) and np.array_equal(v2, vel) and np.array_equal(s2, sp)
        for off in (snapshot.HEADER.size + 3, len(buf) - 1):
            bad = bytearray(buf)
            bad[off] ^= 0x10
            with pytest.raises(ValueError):
                snapshot.unpack(bytes(bad))
        with pytest.raises(ValueError):
            snapshot.unpack(b"XXXXXXXX" + buf[8:])


def test_header_constants_match_the_python_mirror():
    """Every plain #define GBMD_<NAME> <integer> of the header has the same value in _abi as <NAME>,
    and the two flag-field helpers place their values where the header's macros do."""
    text = open(_abi.HEADER_PATH).read()
    found = 0
    for name, value in re.findall(r"#define GBMD_([A-Z0-9_]+) \(?(-?\d+)u?\)?", text):
        if not hasattr(_abi, name):
            continue
        assert getattr(_abi, name) == int(value), name
        found += 1
    assert found >= 20
    assert "#define GBMD_FLAG_BUILD_LANES(s) ((uint32_t)(s) << 4)" in text and _abi.build_lanes_flag(8) == 8 << 4
    assert "#define GBMD_FLAG_FORCE_LANES(s) ((uint32_t)(s) << 8)" in text and _abi.force_lanes_flag(16) == 16 << 8
    with pytest.raises(ValueError):
        _abi.force_lanes_flag(3)


def test_heat_bath_builders_and_validation(engine_lib):
    """The Andersen bath's host side: md-core's builders (with_thermostat keeps a fan's species,
    region and drift; with_fan / with_bath_layer need a thermostat first), the C struct fields,
    and gbmd_create refusing a bad bath before any device work (runs without a GPU)."""
    from micrographia_gb300 import ONE, Pair, System, System3, box_for, cube_for

    s = System(box_for(200, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0, 2.0])
    with pytest.raises(ValueError):
        s.with_fan(0b1, 1.0, 2.0, 0.1)
    s.with_thermostat(0.8, 1.0).with_fan(0b10, 1.5, 4.5, 0.3).with_thermostat(1.1, 2.0)
    th = s.thermostat
    assert (th.t, th.rate, th.species, th.axis, th.drift) == (1.1, 2.0, 0b10, 0, 0.3)
    assert th.region == (int(1.5 * ONE), int(4.5 * ONE))
    c = s.to_c()
    assert (c.bath, c.bath_species, c.bath_axis, c.bath_t, c.bath_rate, c.bath_drift) == (1, 0b10, 0, 1.1, 2.0, 0.3)
    assert list(c.bath_region) == [int(1.5 * ONE), int(4.5 * ONE)]
    s.with_bath_layer(0.0, 3.0)
    assert s.thermostat.axis == 1 and s.thermostat.acts_on(1, [0, 2 * ONE]) and not s.thermostat.acts_on(0, [0, 2 * ONE])
    s3 = System3(cube_for(300, 0.8), 0.005, Pair.lj(2.5), [1.0]).with_thermostat(1.0, 1.0)
    c3 = s3.to_c()
    assert c3.bath == 1 and c3.bath_species == 0xFFFFFFFF and list(c3.bath_region) == [-(1 << 63), (1 << 63) - 1]
    plain = System(box_for(200, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0])
    assert plain.to_c().bath == 0 and plain.deterministic() and not s.deterministic() and not s3.deterministic()
    assert plain.periodic(0) and plain.periodic(1) and not plain.periodic(2) and s3.periodic(2)

    n = 4
    pos = np.zeros((n, 2), np.int64)
    vel = np.zeros((n, 2), np.int32)
    sp = np.zeros(n, np.uint32)
    P = lambda a, t: a.ctypes.data_as(C.POINTER(t))
    for field, value in (("bath_rate", -1.0), ("bath_t", float("nan")), ("bath_axis", 2), ("bath_drift", float("inf"))):
        bad = System(box_for(200, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0]).with_thermostat(1.0, 1.0).to_c()
        setattr(bad, field, value)
        h = C.c_void_p()
        rc = engine_lib.gbmd_create(C.byref(bad), P(pos, C.c_int64), P(vel, C.c_int32), P(sp, C.c_uint32), n, None, C.byref(h))
        assert rc == _abi.E_INVALID, field
        assert b"bath" in engine_lib.gbmd_last_error(), field


def test_walls_builders_and_the_engine_checks(engine_lib):
    """with_walls clears the axis's periodic bit and records each side's kind (and a thermal
    wall's kT); periodic / deterministic / has_soft_walls follow md-core. The GPU engine checks
    the walls before any device work: a walled axis needs a wall kind on each side and a thermal
    wall a finite kT >= 0; a membrane and compartments need a walled axis."""
    from micrographia_gb300 import Pair, System, System3, Wall, box_for, cube_for

    s = System(box_for(200, 0.5, 1.0), 0.005, Pair.wca(), [1.0]).with_walls(1, Wall.soft(), Wall.thermal(1.5))
    c = s.to_c()
    assert c.periodic == 0b01 and list(c.wall_kind[1]) == [_abi.WALL_SOFT, _abi.WALL_THERMAL] and list(c.wall_t[1]) == [0.0, 1.5]
    assert s.periodic(0) and not s.periodic(1) and s.has_soft_walls() and not s.deterministic()
    s3 = System3(cube_for(300, 0.8), 0.005, Pair.wca(), [1.0]).with_walls(2, Wall.hard(), Wall.hard())
    assert s3.to_c().periodic == 0b011 and s3.deterministic() and not s3.has_soft_walls()
    n = 4
    pos = np.full((n, 2), 1 << 33, np.int64)
    vel = np.zeros((n, 2), np.int32)
    sp = np.zeros(n, np.uint32)
    P = lambda a, t: a.ctypes.data_as(C.POINTER(t))
    h = C.c_void_p()
    bad = s.to_c()
    bad.wall_t[1][1] = -1.0
    rc = engine_lib.gbmd_create(C.byref(bad), P(pos, C.c_int64), P(vel, C.c_int32), P(sp, C.c_uint32), n, None, C.byref(h))
    assert rc == _abi.E_INVALID and b"thermal wall" in engine_lib.gbmd_last_error()
    bad = s.to_c()
    bad.wall_kind[1][0] = 0
    rc = engine_lib.gbmd_create(C.byref(bad), P(pos, C.c_int64), P(vel, C.c_int32), P(sp, C.c_uint32), n, None, C.byref(h))
    assert rc == _abi.E_INVALID and b"wall" in engine_lib.gbmd_last_error()
    # a membrane needs walls on its axis (system.rs:259-265); the engine refuses membranes
    with pytest.raises(ValueError):
        System(box_for(200, 0.5, 1.0), 0.005, Pair.wca(), [1.0]).with_membrane(0, 5.0, [0])
    m = System(box_for(200, 0.5, 2.0), 0.005, Pair.wca(), [1.0, 1.0]).with_walls(0, Wall.soft(), Wall.soft())
    m.with_membrane(0, 8.0, [1]).with_pores(2, 0.5)
    cm = m.to_c()
    assert (cm.membrane, cm.membrane_axis, cm.membrane_blocks, cm.membrane_pore_shift) == (1, 0, 0b10, 34)
    cm.periodic = 0b11  # a membrane lies across a walled axis
    rc = engine_lib.gbmd_create(C.byref(cm), P(pos, C.c_int64), P(vel, C.c_int32), P(sp, C.c_uint32), n, None, C.byref(h))
    assert rc == _abi.E_INVALID and b"membrane" in engine_lib.gbmd_last_error()
    # compartments need walls and whole boxes (system.rs:233-241); the engine refuses them
    from micrographia_gb300 import ONE

    box = System([32 * ONE, 32 * ONE], 0.005, Pair.wca(), [1.0])
    with pytest.raises(ValueError):
        box.with_compartments(0, 3)
    box.with_walls(0, Wall.hard(), Wall.hard())
    with pytest.raises(ValueError):
        box.with_compartments(0, 6)  # 64 sigma boxes do not divide 32 sigma
    box.with_compartments(0, 3).with_diathermal_compartments()
    cc = box.to_c()
    assert list(cc.compartments) == [35, 0] and cc.compartments_diathermal == 1
    assert box.compartment_counts() == [4, 1] and box.compartment_of([17 * ONE, 3 * ONE]) == [2, 0]
    cc.periodic = 0b11  # compartments split a walled axis
    rc = engine_lib.gbmd_create(C.byref(cc), P(pos, C.c_int64), P(vel, C.c_int32), P(sp, C.c_uint32), n, None, C.byref(h))
    assert rc == _abi.E_INVALID and b"compartment" in engine_lib.gbmd_last_error()


def test_static_binning_rejects_bad_grids_before_any_device_work(engine_lib):
    """gbmd_bin_cells_static validates its arguments on the host: a cell grid whose product
    wraps modulo 2^64 (2^22 x 2^22 x 2^20), a product of 2^32 - 1 or more, and a box length that
    is not positive are each rejected with GBMD_E_INVALID before any CUDA call (so this runs
    without a GPU; the device pointers are never touched)."""
    from micrographia_gb300 import Pair, System, System3, box_for, cube_for

    fake = C.c_void_p(16)
    s3 = System3(cube_for(1000, 0.8), 0.005, Pair.lj(2.5), [1.0]).to_c()
    for cells in [(1 << 22, 1 << 22, 1 << 20), (1 << 16, 1 << 16, 1), (70000, 70000, 1)]:
        grid = (C.c_uint32 * 3)(*cells)
        rc = engine_lib.gbmd_bin_cells_static(C.byref(s3), fake, 1000, grid, fake, fake, fake, None)
        assert rc == _abi.E_INVALID, cells
        assert b"too many cells" in engine_lib.gbmd_last_error()
    s2 = System(box_for(1000, 0.7, 1.0), 0.005, Pair.lj(2.5), [1.0])
    c2 = s2.to_c()
    c2.box_len[1] = 0
    grid = (C.c_uint32 * 3)(10, 10, 1)
    assert engine_lib.gbmd_bin_cells_static(C.byref(c2), fake, 1000, grid, fake, fake, fake, None) == _abi.E_INVALID
    assert b"box" in engine_lib.gbmd_last_error()


def test_new_entry_points_reject_bad_arguments_on_the_host(engine_lib):
    """The Observer, kinetic-energy and velocity entry points check their arguments before any
    device work: a null engine or system, and species out of range or fixed_speed in 3D."""
    lib = _abi.lib()
    assert lib.gbmd_observe_grid(None, 4, 4, 0, None, None, None) == _abi.E_INVALID
    assert lib.gbmd_read_kinetic(None, None, None, None) == _abi.E_INVALID
    assert lib.gbmd_maxwell(None, None, 0, 1.0, 1, None) == _abi.E_INVALID
    from micrographia_gb300 import Pair, System, System3, box_for, cube_for

    sys2 = System(box_for(100, 0.5, 1.0), 0.005, Pair.lj(2.5), [1.0]).to_c()
    sp = (C.c_uint32 * 2)(0, 3)  # species 3 of a one-species system
    vel = (C.c_int32 * 4)()
    assert lib.gbmd_maxwell(C.byref(sys2), sp, 2, 1.0, 1, vel) == _abi.E_INVALID
    sys3 = System3(cube_for(100, 0.5), 0.005, Pair.lj(2.5), [1.0]).to_c()
    assert lib.gbmd_fixed_speed(C.byref(sys3), (C.c_uint32 * 1)(0), 1, 1.0, 1, (C.c_int32 * 3)()) == _abi.E_UNSUPPORTED
