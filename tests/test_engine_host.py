"""The full-engine worker (engine_core.cuh) compiled for the host, one
worker, against the reference's own alphabeta_gpu kernel on the host
(refshim): through iterative deepening with the tables, killer and counter
moves kept between depths (src/search.c:77-198), every PV slot, the score
and the node / TT-move / TT-score / IID-move counters are equal -- the bar
of the GPU tests, checked without a GPU on the same source."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle_lib as ol

HERE = os.path.dirname(os.path.abspath(__file__))
E1, E2 = 1 << 16, 1 << 14  # TT1 / TT2 entries of both searches
SLOTS = [1, 3, 4, 5]       # nodes, TT-move hits, TT-score hits, IID-move hits

_u64p = ctypes.POINTER(ctypes.c_uint64)
_u32p = ctypes.POINTER(ctypes.c_uint32)


@pytest.fixture(scope="module")
def host_engine(tmp_path_factory):
    if ol.reference() is None:
        pytest.skip("reference kernels (oracle/_ref) not built")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    so = str(tmp_path_factory.mktemp("engine_host") / "libengine_host.so")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-x", "cu", "-Xcompiler", "-fPIC", "-shared", "-o", so,
                    os.path.join(HERE, "host", "engine_host.cu")], check=True)
    lib = ctypes.CDLL(so)
    lib.he_new.restype = ctypes.c_void_p
    lib.he_new.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
    lib.he_free.argtypes = [ctypes.c_void_p]
    lib.he_run.argtypes = [ctypes.c_void_p, _u64p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _u64p,
                           ctypes.c_uint64, _u32p, _u64p]
    return lib


def _compare(lib, board, stm, max_depth, ply_init=0, hist=None):
    ref = ol.RefSearch(E1, E2)
    h = lib.he_new(E1, E2)
    b = np.ascontiguousarray(np.asarray(board, dtype=np.uint64).reshape(7))
    hh = np.zeros(1024, dtype=np.uint64)
    if hist is None:
        hh[ply_init] = b[5]
    else:
        hh[:] = np.asarray(hist, dtype=np.uint64)
    try:
        for d in range(1, max_depth + 1):
            pv_r, c_r = ref.run(b, stm, d, ply_init, hist)
            pv = np.zeros(64, dtype=np.uint32)
            c = np.zeros(64, dtype=np.uint64)
            lib.he_run(h, b.ctypes.data_as(_u64p), int(stm), d, ply_init, hh.ctypes.data_as(_u64p), 1 << 40,
                       pv.ctypes.data_as(_u32p), c.ctypes.data_as(_u64p))
            assert list(pv) == list(pv_r), (d, [ol.move2can(int(m)) for m in pv[1:6]],
                                            [ol.move2can(int(m)) for m in pv_r[1:6]])
            assert [int(c[k]) for k in SLOTS] == [int(c_r[0, k]) for k in SLOTS], d
    finally:
        lib.he_free(h)


def test_initial_position_matches_reference(host_engine):
    b, stm = ol.setboard("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    _compare(host_engine, b, stm, 5)


@pytest.mark.parametrize("fen,depth", [
    ("6k1/5ppp/8/8/8/8/5PPP/3R2K1 w - - 0 1", 5),             # mate in one behind a back rank
    ("8/8/8/8/8/5k2/3p4/5K2 b - - 0 1", 6),                  # promotion: extension, queen moves
    ("8/2p5/3p4/KP5r/1R3p1k/8/4P1P1/8 w - - 0 1", 5),         # pawn endgame, pins
    ("r3k2r/p1ppqpb1/bn2pnp1/3PN3/1p2P3/2N2Q1p/PPPBBPPP/R3K2R w KQkq - 0 1", 3),  # castles, pins
    ("4k3/8/8/8/8/8/8/4K2R w K - 0 1", 6),                   # rook mate: null move, IID, LMR
    ("7k/5Q2/6K1/8/8/8/8/8 b - - 0 1", 3),                   # stalemate
])
def test_special_positions_match_reference(host_engine, fen, depth):
    b, stm = ol.setboard(fen)
    _compare(host_engine, b, stm, depth)


@pytest.mark.parametrize("i", range(12))
def test_workload_positions_match_reference(host_engine, i):
    boards, stm, _ = ol.make_positions(0x5A17A0000000005, 12, min_plies=20, max_plies=40, min_pieces=20,
                                       min_depth=0, max_depth=0)
    _compare(host_engine, boards[i], int(stm[i]), 5)


@pytest.mark.parametrize("i", range(8))
def test_playout_positions_match_reference(host_engine, i):
    """Playouts of 1-150 plies: openings, middlegames and endgames."""
    boards, stm, _ = ol.make_positions(0x77C1, 8, min_plies=1, max_plies=150, min_pieces=0, min_depth=0,
                                       max_depth=0)
    _compare(host_engine, boards[i], int(stm[i]), 5)


def test_repetition_history_matches_reference(host_engine):
    """The initial position reached again after four knight moves: the
    search sees the earlier occurrences through the hash history."""
    b, stm = ol.setboard("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    hist = np.zeros(1024, dtype=np.uint64)
    cur, s = b.copy(), stm
    hist[0] = cur[5]
    for ply, can in enumerate(["g1f3", "g8f6", "f3g1", "f6g8"], start=1):
        cur = ol.play(cur, s, ol.can2move(cur, s, can))
        s ^= 1
        hist[ply] = cur[5]
    _compare(host_engine, cur, s, 4, ply_init=4, hist=hist)
