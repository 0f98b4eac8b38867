"""wfs_observe_noalloc: observables for callers that may not allocate device memory.

Some callers cannot let a library call cudaMalloc: their host application's
allocator owns the GPU's memory, or they run in a loop where an allocation's
locks and implicit synchronisation are not acceptable, or they only receive
device pointers. wfs_observe_noalloc serves them: it reads a psi the caller
owns, writes the observables into a device buffer the caller owns, and keeps
its scratch in a fixed device array inside the library.

These tests call it through the C ABI and compare it with wfs_observe (the
handle-based entry point, which allocates its scratch) on two calls in a row,
with the expected location alone, on a grid that needs exactly as many partial
sums as the fixed scratch holds (also against the oracle's Simpson sums), and
check that one more row of blocks, or a grid far too large, is refused.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, psi_ptr, dtype, n, extent, boxes, loc, out_ptr, stream):
    from wavefunctionsimpython_gb300._lib import Box, make_box

    nb = len(boxes)
    arr = (Box * max(nb, 1))()
    for i, (b, c) in enumerate(boxes):
        arr[i] = make_box(b, c)
    lb = make_box(*loc) if loc is not None else None
    return lib.wfs_observe_noalloc(C.c_void_p(psi_ptr), dtype, (C.c_int32 * 3)(*n), (C.c_double * 3)(*extent),
                                   arr, nb, C.byref(lb) if lb is not None else None,
                                   C.cast(C.c_void_p(out_ptr), C.POINTER(C.c_double)), C.c_void_p(stream))


@pytest.mark.parametrize("dbl", [False, True])
def test_noalloc_matches_observe_twice(dbl):
    import torch

    from wavefunctionsimpython_gb300 import Engine
    from wavefunctionsimpython_gb300._lib import WFS_C64, WFS_C128, WFS_OK, load

    lib = load()
    n, L = (48, 32, 64), (24.0, 16.0, 32.0)
    # one explicit stream orders the engine's work and the allocation-free call
    stream = torch.cuda.Stream()
    assert stream.cuda_stream != 0
    e = Engine(n, L, double_precision=dbl, stream=stream.cuda_stream)
    e.add_wall(3.0, (0, 0, 0), (1, 0, 0), 2.0)
    e.init_gaussian((2.0, 1.5, 2.5), (-3.0, 0.5, 1.0), (1.5, 0.0, 0.5))
    dtype = WFS_C128 if dbl else WFS_C64
    calls = [
        ([((0, 0, 0), (47, 31, 63)), ((24, 1, 3), (23, 29, 57))], ((2, 1, 4), (43, 29, 57))),
        ([((10, 0, 0), (3, 31, 63)), ((0, 0, 0), (1, 1, 1)), ((5, 7, 9), (33, 17, 41))], None),
    ]
    out = torch.full((16,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for k, (boxes, loc) in enumerate(calls):
        if k:
            e.step_split(5, 0.02, 1.0)
        psi_ptr = e.psi_device_ptr()
        with torch.cuda.stream(stream):
            out.fill_(float("nan"))
        rc = _call(lib, psi_ptr, dtype, n, L, boxes, loc, out.data_ptr(), stream.cuda_stream)
        assert rc == WFS_OK, lib.wfs_global_error().decode()
        stream.synchronize()
        got = out.cpu().numpy()
        probs, er, er2 = e.observe(boxes, loc)
        nb = len(boxes)
        np.testing.assert_allclose(got[:nb], probs, rtol=1e-12, atol=0)
        if loc is not None:
            np.testing.assert_allclose(got[nb:nb + 3], er, rtol=1e-12, atol=1e-15)
            np.testing.assert_allclose(got[nb + 3:nb + 6], er2, rtol=1e-12, atol=0)
    e.close()


def test_noalloc_rejects_grid_beyond_scratch():
    import torch

    from wavefunctionsimpython_gb300._lib import WFS_C64, WFS_ERR_UNSUPPORTED, load

    lib = load()
    out = torch.zeros(16, dtype=torch.float64, device="cuda")
    dummy = torch.zeros(8, dtype=torch.complex64, device="cuda")
    # 1024 x 1024 rows / 8 rows per block * 15 quantities far exceeds the fixed scratch;
    # the size check runs before any memory is touched
    n = (1024, 1024, 8)
    boxes = [((0, 0, 0), (1, 1, 1))] * 8
    rc = _call(lib, dummy.data_ptr(), WFS_C64, n, (1.0, 1.0, 1.0), boxes, ((0, 0, 0), (1, 1, 1)),
               out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == WFS_ERR_UNSUPPORTED
    assert b"scratch" in lib.wfs_global_error()


def test_noalloc_location_only_and_exact_scratch_limit():
    """nbox = 0 with a location box (7 quantities), then a (16, 8191, 2) grid with one box
    and a location box: ceil(16 * 8191 / 8) * 8 = 131056 partial sums, exactly what the
    fixed scratch holds (accepted, checked against wfs_observe and the FP64 oracle); a
    (16, 8192, 2) grid needs 131072 and is refused before anything is launched."""
    import torch

    from oracle import wfs_oracle as orc
    from wavefunctionsimpython_gb300 import Engine
    from wavefunctionsimpython_gb300._lib import WFS_C64, WFS_ERR_UNSUPPORTED, WFS_OK, load

    lib = load()
    stream = torch.cuda.Stream()
    out = torch.full((16,), float("nan"), dtype=torch.float64, device="cuda")

    # location only
    n, L = (40, 24, 32), (20.0, 12.0, 16.0)
    e = Engine(n, L, stream=stream.cuda_stream)
    e.init_gaussian((2.0, 1.5, 2.0), (-2.0, 1.0, 0.5), (1.0, 0.0, 0.5))
    loc = ((1, 2, 3), (37, 19, 27))
    torch.cuda.synchronize()
    rc = _call(lib, e.psi_device_ptr(), WFS_C64, n, L, [], loc, out.data_ptr(), stream.cuda_stream)
    assert rc == WFS_OK, lib.wfs_global_error().decode()
    stream.synchronize()
    got = out.cpu().numpy()
    _, er, er2 = e.observe([], loc)
    np.testing.assert_allclose(got[0:3], er, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(got[3:6], er2, rtol=1e-12, atol=0)
    e.close()

    # exactly at the limit
    n, L = (16, 8191, 2), (8.0, 4095.5, 1.0)
    e = Engine(n, L, stream=stream.cuda_stream)
    rng = np.random.default_rng(11)
    psi = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    e.set_psi(psi)
    boxes = [((1, 10, 0), (13, 8001, 1))]
    loc = ((0, 0, 0), (15, 8191, 1))
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        out.fill_(float("nan"))
    rc = _call(lib, e.psi_device_ptr(), WFS_C64, n, L, boxes, loc, out.data_ptr(), stream.cuda_stream)
    assert rc == WFS_OK, lib.wfs_global_error().decode()
    stream.synchronize()
    got = out.cpu().numpy()
    probs, er, er2 = e.observe(boxes, loc)
    np.testing.assert_allclose(got[:1], probs, rtol=1e-12, atol=0)
    np.testing.assert_allclose(got[1:4], er, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(got[4:7], er2, rtol=1e-12, atol=0)
    dx = orc.delta_x(L, n)
    np.testing.assert_allclose(got[0], orc.volume_probability(psi, dx, *boxes[0]), rtol=1e-6)
    oer, oer2 = orc.expected_location(psi, dx, *loc)
    np.testing.assert_allclose(got[1:4], oer, rtol=1e-5, atol=1e-6 * float(np.max(np.abs(oer2))) ** 0.5)
    np.testing.assert_allclose(got[4:7], oer2, rtol=1e-6)
    e.close()

    # one block row more than the scratch holds
    dummy = torch.zeros(8, dtype=torch.complex64, device="cuda")
    rc = _call(lib, dummy.data_ptr(), WFS_C64, (16, 8192, 2), (8.0, 4096.0, 1.0), boxes, loc, out.data_ptr(),
               stream.cuda_stream)
    assert rc == WFS_ERR_UNSUPPORTED
    assert b"131072" in lib.wfs_global_error()
