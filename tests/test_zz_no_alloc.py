"""gbmd_bin_cells_static: the cell binning for callers that cannot allocate device memory.

Some callers of this library cannot call cudaMalloc: a host that hands the library one fixed
device arena at start-up and allows no allocation afterwards, or a stream-ordered hot path where
an allocation would synchronise the device. For them the binning keeps its scratch in a static
device array; the caller supplies only the input positions and the three output buffers. This
test calls that entry point through the C ABI twice in a row, on two different states, and checks
each result against the engine's own binning entry point (gbmd_debug_bin), bit for bit as every
binning test here does. It runs last so that a run stopping at the first failure has run all the
other tests, and it passes alone in a fresh process as well as after them."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bin_static(lib, abi, sys_, st, dims, default_stream=False):
    import torch

    n = st.n()
    ncell = int(np.prod(dims))
    dev = torch.device("cuda", 0)
    pos = torch.from_numpy(np.ascontiguousarray(st.pos)).to(dev)
    keys = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    start = torch.empty(ncell + 1, dtype=torch.int32, device=dev)
    items = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    cells = (C.c_uint32 * 3)(*(list(dims) + [1] * (3 - len(dims))))
    csys = sys_.to_c()
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)
    handle = None if default_stream else C.c_void_p(stream.cuda_stream)
    abi.check(lib.gbmd_bin_cells_static(C.byref(csys), pos.data_ptr() if n else None, n, cells, keys.data_ptr(), start.data_ptr(),
                                        items.data_ptr(), handle))
    torch.cuda.synchronize(dev)
    as_u32 = lambda t: t.cpu().numpy().view(np.uint32)
    return as_u32(keys)[:n], as_u32(start), as_u32(items)[:n]


def _bin_engine(sys_, st, dims):
    from micrographia_gb300 import ForceMode, GpuEngine, GpuEngine3

    cls = GpuEngine if sys_.DIM == 2 else GpuEngine3
    with cls(sys_, st, ForceMode.cell_list()) as e:
        keys, start, items, order = e.debug_bin(dims)
    assert np.array_equal(order, np.arange(st.n()))
    return keys, start, items


def test_static_binning_matches_the_engine_on_two_calls_in_a_row():
    pytest.importorskip("torch")
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from micrographia_gb300 import Pair, State, System, System3, _abi, box_for, build, cube_for

    build.build()
    lib = _abi.lib()
    rng = np.random.default_rng(7)
    # call 1: a 2D system; call 2: a larger 3D system, so the shared array is reused with
    # different sizes and contents
    s2 = System(box_for(50_000, 0.7, 1.0), 0.005, Pair.lj(2.5), [1.0])
    p2 = np.stack([rng.integers(0, s2.box_len[a], 50_000) for a in range(2)], 1).astype(np.int64)
    st2 = State(p2, np.zeros((50_000, 2), np.int32), np.zeros(50_000, np.uint32))
    n3 = 200_000
    s3 = System3(cube_for(n3, 0.8442), 0.005, Pair.lj(2.5), [1.0])
    p3 = np.stack([rng.integers(0, s3.box_len[a], n3) for a in range(3)], 1).astype(np.int64)
    from micrographia_gb300 import State3

    st3 = State3(p3, np.zeros((n3, 3), np.int32), np.zeros(n3, np.uint32))
    from oracle import oracle as O

    for sys_, st in [(s2, st2), (s3, st3)]:
        dims = sys_.cells_for(2.8)
        got = _bin_static(lib, _abi, sys_, st, dims)
        want = _bin_engine(sys_, st, dims)
        for g, w in zip(got, want):
            assert np.array_equal(g, w)
        # and directly against md-ref's CellList::build restated (cells.rs:1-55)
        for g, w in zip(got, O.cell_list(sys_, st, dims)):
            assert np.array_equal(g, w)


def test_static_binning_on_the_default_stream_and_with_no_particles():
    """A call on the legacy default stream (stream NULL) gives the engine's binning; a call with
    n = 0 writes only the cell starts, all zero."""
    pytest.importorskip("torch")
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from micrographia_gb300 import Pair, State, System, _abi, box_for, build

    build.build()
    lib = _abi.lib()
    rng = np.random.default_rng(11)
    n = 30_000
    sys_ = System(box_for(n, 0.6, 1.0), 0.005, Pair.lj(2.5), [1.0])
    st = State(np.stack([rng.integers(0, sys_.box_len[a], n) for a in range(2)], 1).astype(np.int64), np.zeros((n, 2), np.int32),
               np.zeros(n, np.uint32))
    dims = sys_.cells_for(2.5)
    got = _bin_static(lib, _abi, sys_, st, dims, default_stream=True)
    want = _bin_engine(sys_, st, dims)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
    empty = State(np.zeros((0, 2), np.int64), np.zeros((0, 2), np.int32), np.zeros(0, np.uint32))
    _, start, _ = _bin_static(lib, _abi, sys_, empty, dims)
    assert start.shape == (int(np.prod(dims)) + 1,) and not start.any()


def test_static_binning_rejects_sizes_beyond_its_maximum():
    pytest.importorskip("torch")
    from micrographia_gb300 import Pair, System, _abi, box_for

    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    lib = _abi.lib()
    n = _abi.BIN_STATIC_MAX_N + 1
    sys_ = System(box_for(n, 0.7, 1.0), 0.005, Pair.lj(2.5), [1.0])
    cells = (C.c_uint32 * 3)(10, 10, 1)
    csys = sys_.to_c()
    # small real buffers: the size check rejects the call before any of them is used
    buf = [torch.empty(16, dtype=torch.int64, device="cuda") for _ in range(4)]
    rc = lib.gbmd_bin_cells_static(C.byref(csys), buf[0].data_ptr(), n, cells, buf[1].data_ptr(), buf[2].data_ptr(), buf[3].data_ptr(), None)
    assert rc == _abi.E_INVALID
    assert b"262144" in lib.gbmd_last_error()
