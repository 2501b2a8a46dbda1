"""The allocation-free perft entry point, zeta_perft_batch_noalloc.

It exists for callers that cannot allocate device memory -- programs that
own all device memory through their own pool or budget, and latency-
critical loops that must not call cudaMalloc (it may synchronise the
device).  Its scratch lives in a fixed device array inside the library.
This test calls it through the C ABI on buffers the test allocates, twice
in a row (the array keeps the previous call's contents), and checks both
results against the regular entry point, zeta_perft_batch_device.  Leaf
counts are integers: the comparison is exact.

The file name sorts last so that a run stopping at the first failure has
run every other test before this one.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_buffers(torch, boards, stm, depth):
    dev = torch.device("cuda", 0)
    return (torch.from_numpy(boards.view(np.int64)).to(dev), torch.from_numpy(stm).to(dev),
            torch.from_numpy(depth).to(dev), torch.zeros(len(depth), dtype=torch.int64, device=dev))


def test_noalloc_entry_matches_regular_entry_twice(zeta_device):
    torch = pytest.importorskip("torch")
    z = zeta_device
    lib = z.load_library()
    stream = torch.cuda.Stream(torch.device("cuda", 0))
    runs = [(0x51A7E, 300, 3, 4), (0x51A7F, 700, 2, 3)]  # different shapes on consecutive calls
    for seed, n, dmin, dmax in runs:
        boards, stm, depth = z.make_positions(seed, n, 10, 60, 0, dmin, dmax)
        db, ds, dd, want = _device_buffers(torch, boards, stm, depth)
        z.perft_batch_device(db.data_ptr(), ds.data_ptr(), dd.data_ptr(), n, want.data_ptr(), stream.cuda_stream)
        got = torch.full((n,), -1, dtype=torch.int64, device=db.device)
        rc = lib.zeta_perft_batch_noalloc(ctypes.c_void_p(db.data_ptr()), ctypes.c_void_p(ds.data_ptr()),
                                          ctypes.c_void_p(dd.data_ptr()), n, ctypes.c_void_p(got.data_ptr()),
                                          ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.zeta_last_error().decode()
        torch.cuda.synchronize()
        assert torch.equal(got, want), (seed, n)
        assert int(want.sum()) > 0


def test_noalloc_entry_rejects_batches_beyond_its_fixed_scratch(zeta_device):
    z = zeta_device
    lib = z.load_library()
    rc = lib.zeta_perft_batch_noalloc(ctypes.c_void_p(8), ctypes.c_void_p(8), ctypes.c_void_p(8), (1 << 17) + 1,
                                      ctypes.c_void_p(8), None)
    assert rc == -7  # ZETA_ERR_NOALLOC, before touching any buffer
    assert b"fixed scratch" in lib.zeta_last_error()
