"""The caller-buffer Life entry point that allocates nothing.

om_life_proceed_noalloc is for callers that cannot call cudaMalloc: a host
framework whose allocator owns all device memory, or a real-time loop that
must not block on the allocator.  Here the test, acting as such a caller,
owns the grids; the entry point's only scratch is a fixed device array shared
by all calls.  Its results must equal the regular handle-based path and the
oracle, call after call.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    f = lib.om_life_proceed_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    return f


def test_noalloc_matches_handle_path_twice(om_lib):
    import torch
    pg = om_lib
    lib = pg.load_library()
    f = _noalloc(lib)
    n0, n1 = 2048, 768
    ref = pg.Life((n0, n1))
    ref.fill_random(21, 0.3)
    init = ref.read("cell")
    # caller-owned device grids (allocated by the caller, not by the call)
    a = torch.from_numpy(init.copy()).cuda()
    b = torch.empty_like(a)
    c = torch.empty_like(a)
    torch.cuda.synchronize()
    pops1 = np.zeros(32, np.int32)
    pops2 = np.zeros(7, np.int32)
    # first call: 32 generations a -> b (pops to host memory)
    assert f(a.data_ptr(), b.data_ptr(), n0, n1, 32, pops1.ctypes.data, None) == 0, \
        lib.om_last_error()
    ref.proceed(32)
    assert np.array_equal(b.cpu().numpy(), ref.read("cell"))
    assert np.array_equal(pops1, ref.population_history(32))
    # second call in a row: 7 generations b -> c, populations to device memory
    dpops = torch.zeros(7, dtype=torch.int32, device="cuda")
    assert f(b.data_ptr(), c.data_ptr(), n0, n1, 7, dpops.data_ptr(), None) == 0, \
        lib.om_last_error()
    pops2[:] = dpops.cpu().numpy()
    ref.proceed(7)
    assert np.array_equal(c.cpu().numpy(), ref.read("cell"))
    assert np.array_equal(pops2, ref.population_history(7))
    ref.close()


def test_noalloc_rejects_out_of_range(om_lib):
    import torch
    lib = om_lib.load_library()
    f = _noalloc(lib)
    a = torch.zeros(64 * 8, dtype=torch.int32, device="cuda")
    b = torch.zeros_like(a)
    pops = np.zeros(64, np.int32)
    assert f(a.data_ptr(), b.data_ptr(), 64, 8, 33, pops.ctypes.data, None) == 1
    assert b"generations must be in [1, 32]" in lib.om_last_error()
    assert f(a.data_ptr(), b.data_ptr(), 48, 8, 4, pops.ctypes.data, None) == 1
    assert f(a.data_ptr(), a.data_ptr(), 64, 8, 4, pops.ctypes.data, None) == 1
    a[5] = 2                                  # not a Life cell value
    assert f(a.data_ptr(), b.data_ptr(), 64, 8, 4, pops.ctypes.data, None) == 1
    assert b"0 or 1" in lib.om_last_error()


@pytest.mark.parametrize("n0,n1", [(96, 50), (32, 1), (32, 3), (64, 17), (64, 1)])
def test_noalloc_ragged_and_tiny_grids(om_lib, oracle, n0, n1):
    """Grids whose rows are not a multiple of the 64-row tile, narrower than
    a 32-word tile, or a single row: 1 and then 32 generations, on a
    non-default stream, against the oracle."""
    import torch
    lib = om_lib.load_library()
    f = _noalloc(lib)
    init = oracle.life_bernoulli(n0, n1, 5 + n0 + n1, 0.3)
    a = torch.from_numpy(init.copy()).cuda()
    b = torch.empty_like(a)
    c = torch.empty_like(a)
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    pops1 = np.zeros(1, np.int32)
    pops32 = np.zeros(32, np.int32)
    assert f(a.data_ptr(), b.data_ptr(), n0, n1, 1, pops1.ctypes.data,
             C.c_void_p(stream.cuda_stream)) == 0, lib.om_last_error()
    want1, wpops1 = oracle.life_run(init, 1, cyclic=True)
    assert np.array_equal(b.cpu().numpy(), want1)
    assert np.array_equal(pops1, wpops1)
    assert f(b.data_ptr(), c.data_ptr(), n0, n1, 32, pops32.ctypes.data,
             C.c_void_p(stream.cuda_stream)) == 0, lib.om_last_error()
    want32, wpops32 = oracle.life_run(want1, 32, cyclic=True)
    assert np.array_equal(c.cpu().numpy(), want32)
    assert np.array_equal(pops32, wpops32)


def test_noalloc_rejects_population_overflow(om_lib):
    """More than 2^31 - 1 cells is rejected before any device work (the
    buffers are never touched, so small ones stand in)."""
    import torch
    lib = om_lib.load_library()
    f = _noalloc(lib)
    a = torch.zeros(64, dtype=torch.int32, device="cuda")
    b = torch.zeros_like(a)
    pops = np.zeros(4, np.int32)
    assert f(a.data_ptr(), b.data_ptr(), 1 << 20, 1 << 20, 4, pops.ctypes.data, None) == 1
    assert b"2^31 - 1 cells" in lib.om_last_error()
