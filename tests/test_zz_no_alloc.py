"""The allocation-free perft entry point, zeta_perft_batch_noalloc.

It exists for callers that cannot allocate device memory -- programs that
own all device memory through their own pool or budget, and latency-
critical loops that must not call cudaMalloc (it may synchronise the
device).  Its scratch lives in a fixed device array inside the library.
These tests call it through the C ABI on buffers the test allocates:
twice in a row (the array keeps the previous call's contents) against the
regular entry point, zeta_perft_batch_device; against the reference
kernel's own counts (tests/golden/perft_ref.json); past its fixed task
capacity; and from a fresh process that never calls zeta_init.  Leaf
counts are integers: every comparison is exact.

The file name sorts last so that a run stopping at the first failure has
run every other test before this one.
"""
import ctypes
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
ZETA_ERR_NOALLOC = -7


def _device_buffers(torch, boards, stm, depth):
    dev = torch.device("cuda", 0)
    return (torch.from_numpy(boards.view(np.int64)).to(dev), torch.from_numpy(stm).to(dev),
            torch.from_numpy(depth).to(dev), torch.zeros(len(depth), dtype=torch.int64, device=dev))


def _noalloc(lib, db, ds, dd, n, out, stream):
    return lib.zeta_perft_batch_noalloc(ctypes.c_void_p(db.data_ptr()), ctypes.c_void_p(ds.data_ptr()),
                                        ctypes.c_void_p(dd.data_ptr()), n, ctypes.c_void_p(out.data_ptr()),
                                        ctypes.c_void_p(stream))


def _golden_random_d3():
    cases = [c for c in json.load(open(os.path.join(HERE, "golden", "perft_ref.json")))
             if c["name"].startswith("random") and c["depth"] == 3]
    boards = np.array([[int(x, 16) for x in c["board"]] for c in cases], dtype=np.uint64)
    stm = np.array([c["stm"] for c in cases], dtype=np.uint8)
    depth = np.array([c["depth"] for c in cases], dtype=np.uint8)
    return boards, stm, depth, np.array([c["leaves"] for c in cases], dtype=np.uint64)


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
        rc = _noalloc(lib, db, ds, dd, n, got, stream.cuda_stream)
        assert rc == 0, lib.zeta_last_error().decode()
        torch.cuda.synchronize()
        assert torch.equal(got, want), (seed, n)
        assert int(want.sum()) > 0


def test_noalloc_entry_matches_reference_kernel_counts(zeta_device):
    """The 96 random playout positions at depth 3 whose counts the reference
    perft kernel itself produced (refshim, unmodified zetaperft.cl)."""
    torch = pytest.importorskip("torch")
    lib = zeta_device.load_library()
    boards, stm, depth, want = _golden_random_d3()
    db, ds, dd, out = _device_buffers(torch, boards, stm, depth)
    assert _noalloc(lib, db, ds, dd, len(depth), out, 0) == 0, lib.zeta_last_error().decode()
    assert np.array_equal(out.cpu().numpy().view(np.uint64), want)


def test_noalloc_entry_rejects_batches_beyond_its_fixed_scratch(zeta_device):
    z = zeta_device
    lib = z.load_library()
    rc = lib.zeta_perft_batch_noalloc(ctypes.c_void_p(8), ctypes.c_void_p(8), ctypes.c_void_p(8), (1 << 17) + 1,
                                      ctypes.c_void_p(8), None)
    assert rc == ZETA_ERR_NOALLOC  # before touching any buffer
    assert b"fixed scratch" in lib.zeta_last_error()


def test_noalloc_entry_reports_a_split_beyond_its_task_arrays(zeta_device):
    """256 middlegame positions at depth 5: the second split level would
    hold ~300 K subtree tasks, past the fixed 131,072.  The call stops the
    split at the overflow, runs no subtree and returns ZETA_ERR_NOALLOC;
    the next call on the same array is right again."""
    torch = pytest.importorskip("torch")
    z = zeta_device
    lib = z.load_library()
    boards, stm, _ = z.make_positions(0x0F10, 256, 20, 40, 20, 5, 5)
    depth = np.full(256, 5, dtype=np.uint8)
    db, ds, dd, out = _device_buffers(torch, boards, stm, depth)
    assert _noalloc(lib, db, ds, dd, 256, out, 0) == ZETA_ERR_NOALLOC
    assert b"subtree tasks" in lib.zeta_last_error()
    boards, stm, depth, want = _golden_random_d3()
    db, ds, dd, out = _device_buffers(torch, boards, stm, depth)
    assert _noalloc(lib, db, ds, dd, len(depth), out, 0) == 0, lib.zeta_last_error().decode()
    assert np.array_equal(out.cpu().numpy().view(np.uint64), want)


FRESH = r"""
import ctypes, json, os, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
import zeta_gb300 as z
lib = z.load_library()          # loaded, never initialised: no zeta_init
cases = [c for c in json.load(open(sys.argv[2])) if c["name"].startswith("random") and c["depth"] == 3]
b = torch.tensor(np.array([[int(x, 16) for x in c["board"]] for c in cases], dtype=np.uint64).view(np.int64),
                 device="cuda")
s = torch.tensor([c["stm"] for c in cases], dtype=torch.uint8, device="cuda")
d = torch.tensor([c["depth"] for c in cases], dtype=torch.uint8, device="cuda")
want = np.array([c["leaves"] for c in cases], dtype=np.uint64)
for _ in range(2):
    out = torch.full((len(cases),), -1, dtype=torch.int64, device="cuda")
    rc = lib.zeta_perft_batch_noalloc(ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(s.data_ptr()),
                                      ctypes.c_void_p(d.data_ptr()), len(cases), ctypes.c_void_p(out.data_ptr()),
                                      None)
    assert rc == 0, lib.zeta_last_error().decode()
    assert np.array_equal(out.cpu().numpy().view(np.uint64), want)
print("fresh-ok", len(cases))
"""


def test_noalloc_entry_needs_no_init_in_a_fresh_process():
    pytest.importorskip("torch")
    r = subprocess.run([sys.executable, "-c", FRESH, ROOT, os.path.join(HERE, "golden", "perft_ref.json")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "fresh-ok 96" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]
