"""ctypes bindings of the test oracle (oracle/_build/libzeta_oracle.so) and of
the reference kernels compiled for the host (oracle/_ref/librefzeta.so).

Test infrastructure only: the product never imports this module.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "libzeta_oracle.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "librefzeta.so")

_B7 = ctypes.c_uint64 * 7
_o = None
_r = None


def oracle() -> ctypes.CDLL:
    global _o
    if _o is None:
        if not os.path.exists(ORACLE_SO):
            import subprocess
            subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
        o = ctypes.CDLL(ORACLE_SO)
        o.zo_perft.restype = ctypes.c_uint64
        o.zo_perft_ex.restype = ctypes.c_uint64
        o.zo_computehash.restype = ctypes.c_uint64
        o.zo_splitmix64.restype = ctypes.c_uint64
        o.zo_can2move.restype = ctypes.c_uint32
        for name in ("zo_attack_tables", "zo_pawn_push_tables", "zo_inbetween_table", "zo_line_table"):
            getattr(o, name).restype = ctypes.POINTER(ctypes.c_uint64)
        _o = o
    return _o


def reference():
    """The reference kernels on host cores, or None where they were not built."""
    global _r
    if _r is None and os.path.exists(REF_SO):
        r = ctypes.CDLL(REF_SO)
        r.ref_perft.restype = ctypes.c_uint64
        r.ref_perft_split.restype = ctypes.c_uint64
        r.ref_search_new.restype = ctypes.c_void_p
        r.ref_search_new.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int]
        r.ref_search_free.argtypes = [ctypes.c_void_p]
        r.ref_search_clear.argtypes = [ctypes.c_void_p]
        r.ref_search_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64), ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint32),
                                     ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint32),
                                     ctypes.POINTER(ctypes.c_uint64)]
        _r = r
    return _r


def setboard(fen: str):
    b = _B7()
    stm = ctypes.c_int()
    ok = oracle().zo_setboard(b, ctypes.byref(stm), fen.encode())
    if not ok:
        raise ValueError(f"invalid FEN: {fen}")
    return np.array(list(b), dtype=np.uint64), stm.value


def _b7(board) -> ctypes.Array:
    return _B7(*[int(x) for x in np.asarray(board, dtype=np.uint64).reshape(7)])


def perft(board, stm: int, depth: int, all_promotions: bool = False) -> int:
    if all_promotions:
        return oracle().zo_perft_ex(_b7(board), int(stm), int(depth), 1)
    return oracle().zo_perft(_b7(board), int(stm), int(depth))


def ref_perft(board, stm: int, depth: int, threads: int = 1) -> int:
    r = reference()
    if r is None:
        raise RuntimeError("reference kernels not built")
    if threads > 1:
        return r.ref_perft_split(_b7(board), int(stm), int(depth), threads)
    return r.ref_perft(_b7(board), int(stm), int(depth))


def ref_perft_batch(boards, stm, depth, threads: int) -> np.ndarray:
    r = reference()
    b = np.ascontiguousarray(boards, dtype=np.uint64).reshape(-1, 7)
    n = b.shape[0]
    s = np.ascontiguousarray(stm, dtype=np.int32)
    d = np.ascontiguousarray(depth, dtype=np.int32)
    out = np.zeros(n, dtype=np.uint64)
    r.ref_perft_batch(b.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), s.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                      d.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n,
                      out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), threads)
    return out


class RefSearch:
    """The reference's alphabeta_gpu kernel on the host (refshim), with its
    own transposition tables, killer and counter moves kept between runs as
    the reference keeps its device buffers (src/clrun.c:387-511)."""

    def __init__(self, tt1_entries: int, tt2_entries: int, workers: int = 1):
        self.r = reference()
        if self.r is None:
            raise RuntimeError("reference kernels not built")
        self.workers = workers
        self.h = self.r.ref_search_new(tt1_entries, tt2_entries, workers)

    def run(self, board, stm: int, depth: int, ply_init: int = 0, hist=None, max_nodes: int = 1 << 40):
        """One cl_run_alphabeta launch: (PV uint32[64], counters uint64[workers, 64])."""
        b = _b7(board)
        h = np.zeros(1024, dtype=np.uint64)
        if hist is None:
            h[ply_init] = np.uint64(int(np.asarray(board, dtype=np.uint64).reshape(7)[5]))
        else:
            h[:] = np.asarray(hist, dtype=np.uint64).reshape(1024)
        pv = np.zeros(64, dtype=np.uint32)
        cnt = np.zeros((self.workers, 64), dtype=np.uint64)
        self.r.ref_search_run(self.h, b, int(stm), int(depth), int(ply_init),
                              h.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), None, max_nodes,
                              pv.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                              cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
        return pv, cnt

    def clear(self):
        self.r.ref_search_clear(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.r.ref_search_free(self.h)
            self.h = None


def genmoves(board, stm: int, qs: bool = False, all_promotions: bool = False) -> list[int]:
    buf = (ctypes.c_uint32 * 256)()
    n = oracle().zo_genmoves_ex(_b7(board), int(stm), int(qs), int(all_promotions), buf)
    return list(buf[:n])


def movecount(board, stm: int):
    kic = ctypes.c_int()
    n = oracle().zo_movecount(_b7(board), int(stm), ctypes.byref(kic))
    return n, bool(kic.value)


def play(board, stm: int, move: int, perft_flags: bool = False) -> np.ndarray:
    b = _b7(board)
    oracle().zo_play(b, int(stm), ctypes.c_uint32(move), int(perft_flags))
    return np.array(list(b), dtype=np.uint64)


def computehash(board, stm: int) -> int:
    return oracle().zo_computehash(_b7(board), int(stm))


def eval_white(board) -> int:
    return oracle().zo_eval_white(_b7(board))


def negamax(board, stm: int, depth: int):
    m = ctypes.c_uint32()
    nodes = ctypes.c_uint64()
    v = oracle().zo_negamax(_b7(board), int(stm), int(depth), ctypes.byref(m), ctypes.byref(nodes))
    return v, m.value, nodes.value


def alphabeta(board, stm: int, depth: int):
    m = ctypes.c_uint32()
    nodes = ctypes.c_uint64()
    v = oracle().zo_alphabeta(_b7(board), int(stm), int(depth), ctypes.byref(m), ctypes.byref(nodes))
    return v, m.value, nodes.value


def alphabeta_ordered(board, stm: int, depth: int):
    """The alpha-beta value with reordered moves (same value, fewer nodes)."""
    m = ctypes.c_uint32()
    nodes = ctypes.c_uint64()
    v = oracle().zo_alphabeta_ordered(_b7(board), int(stm), int(depth), ctypes.byref(m), ctypes.byref(nodes))
    return v, m.value, nodes.value


def make_position(seed: int, i: int, min_plies: int, max_plies: int, min_pieces: int, min_depth: int,
                  max_depth: int):
    b = _B7()
    stm = ctypes.c_int()
    depth = ctypes.c_int()
    ok = oracle().zo_make_position(ctypes.c_uint64(seed & (2**64 - 1)), i, min_plies, max_plies, min_pieces,
                                   min_depth, max_depth, b, ctypes.byref(stm), ctypes.byref(depth))
    if not ok:
        return None
    return np.array(list(b), dtype=np.uint64), stm.value, depth.value


def make_positions(seed: int, n: int, **kw):
    boards = np.zeros((n, 7), dtype=np.uint64)
    stm = np.zeros(n, dtype=np.uint8)
    depth = np.zeros(n, dtype=np.uint8)
    for i in range(n):
        r = make_position(seed, i, kw["min_plies"], kw["max_plies"], kw.get("min_pieces", 0),
                          kw.get("min_depth", 0), kw.get("max_depth", 0))
        assert r is not None
        boards[i], stm[i], depth[i] = r
    return boards, stm, depth


def playout(seed: int, plies: int):
    b = _B7()
    stm = ctypes.c_int()
    ok = oracle().zo_playout(ctypes.c_uint64(seed & (2**64 - 1)), plies, b, ctypes.byref(stm))
    return (np.array(list(b), dtype=np.uint64), stm.value) if ok else None


def can2move(board, stm: int, can: str) -> int:
    return int(oracle().zo_can2move(can.encode(), _b7(board), int(stm)))


def move2can(move: int) -> str:
    buf = ctypes.create_string_buffer(6)
    oracle().zo_move2can(ctypes.c_uint32(move), buf)
    return buf.value.decode()


def table(name: str, n: int) -> np.ndarray:
    p = getattr(oracle(), name)()
    return np.ctypeslib.as_array(p, shape=(n,)).copy()
