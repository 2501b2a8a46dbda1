"""zeta_gb300 -- GB300-native device path of the Zeta chess engine.

Python binding of ``libzeta_cuda.so`` (C ABI in ``include/zeta_cuda.h``).
The library is built in-tree by ``zeta_gb300.build`` (``__graft_entry__.build()``);
importing this module does not build anything, and every call fails loudly
when the library or a GB300 is missing -- there is no CPU fallback.

Boards are the reference quad-bitboard (7 x u64, src/types.h:59-66) as numpy
``uint64`` arrays of shape (7,) or (n, 7).
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libzeta_cuda.so")
ROOT = os.path.dirname(_HERE)

ZETA_OK = 0
ERROR_NAMES = {
    -1: "ZETA_ERR_CUDA",
    -2: "ZETA_ERR_ARG",
    -3: "ZETA_ERR_STATE",
    -4: "ZETA_ERR_CAPACITY",
    -5: "ZETA_ERR_DEVICE",
    -6: "ZETA_ERR_BUDGET",
    -7: "ZETA_ERR_NOALLOC",
}


class ZetaError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {message}")
        self.code = code


class PerftConfig(ctypes.Structure):
    _fields_ = [
        ("threads_per_block", ctypes.c_int),
        ("blocks_per_sm", ctypes.c_int),
        ("min_tasks", ctypes.c_uint32),
        ("task_depth", ctypes.c_int),
        ("use_graph", ctypes.c_int),
    ]


class PerftStats(ctypes.Structure):
    _fields_ = [
        ("tasks", ctypes.c_uint64),
        ("steals", ctypes.c_uint64),
        ("interior_nodes", ctypes.c_uint64),
        ("counted_nodes", ctypes.c_uint64),
        ("kernel_ms", ctypes.c_float),
        ("total_ms", ctypes.c_float),
    ]


_u64p = ctypes.POINTER(ctypes.c_uint64)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_i32p = ctypes.POINTER(ctypes.c_int32)

# every symbol include/zeta_cuda.h declares, with its ctypes signature
SIGNATURES = {
    "zeta_init": (ctypes.c_int, [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64]),
    "zeta_release": (ctypes.c_int, []),
    "zeta_last_error": (ctypes.c_char_p, []),
    "zeta_device_info": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                        ctypes.POINTER(ctypes.c_int), _u64p]),
    "zeta_perft": (ctypes.c_int, [_u64p, ctypes.c_int, ctypes.c_int, _u64p]),
    "zeta_perft_batch": (ctypes.c_int, [_u64p, _u8p, _u8p, ctypes.c_int, _u64p]),
    "zeta_perft_batch_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                               ctypes.c_void_p, ctypes.c_void_p]),
    "zeta_perft_batch_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                                ctypes.c_void_p, ctypes.c_void_p]),
    "zeta_perft_configure": (ctypes.c_int, [ctypes.POINTER(PerftConfig)]),
    "zeta_perft_get_config": (ctypes.c_int, [ctypes.POINTER(PerftConfig)]),
    "zeta_perft_set_promotions": (ctypes.c_int, [ctypes.c_int]),
    "zeta_perft_get_promotions": (ctypes.c_int, []),
    "zeta_perft_last_stats": (ctypes.c_int, [ctypes.POINTER(PerftStats)]),
    "zeta_make_positions": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, _u64p, _u8p, _u8p]),
    "zeta_int_peak": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double)]),
    "zeta_search_batch": (ctypes.c_int, [_u64p, _u8p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _u32p, _u64p]),
    "zeta_engine_search": (ctypes.c_int, [_u64p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _u64p, ctypes.c_uint64,
                                          ctypes.c_int, _u32p, _u64p]),
    "zeta_engine_batch": (ctypes.c_int, [_u64p, _u8p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                         _i32p, _u32p, _u64p, _u32p]),
    "zeta_engine_id": (ctypes.c_int, [_u64p, _u8p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                      ctypes.c_int, _i32p, _u32p, _u64p, _u8p, ctypes.POINTER(ctypes.c_float),
                                      ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "zeta_search_batch_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_void_p]),
    "zeta_gemm_configure": (ctypes.c_int, [ctypes.c_int]),
    "zeta_gemm_tc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "zeta_mlp_init": (ctypes.c_int, [ctypes.c_uint64]),
    "zeta_mlp_param_count": (ctypes.c_int, []),
    "zeta_mlp_get_params": (ctypes.c_int, [ctypes.POINTER(ctypes.c_float)]),
    "zeta_mlp_set_params": (ctypes.c_int, [ctypes.POINTER(ctypes.c_float)]),
    "zeta_mlp_grads": (ctypes.c_int, [_u64p, _u8p, _u32p, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                                      ctypes.POINTER(ctypes.c_float)]),
    "zeta_mlp_train": (ctypes.c_int, [_u64p, _u8p, _u32p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                      ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "zeta_mlp_scores": (ctypes.c_int, [_u64p, _u8p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float), _u8p,
                                       _i32p]),
    "zeta_search": (ctypes.c_int, [_u64p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _u64p, ctypes.c_uint64, _u32p,
                                   _u64p]),
    "zeta_search_id": (ctypes.c_int, [_u64p, _u8p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p,
                                      _u32p, _u64p, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                      ctypes.POINTER(ctypes.c_float)]),
    "zeta_search_set_learned_order": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "zeta_tt_clear": (ctypes.c_int, []),
    "zeta_search_set_helpers": (ctypes.c_int, [ctypes.c_int]),
    "zeta_search_set_launch_form": (ctypes.c_int, [ctypes.c_int]),
    "zeta_engine_set_helper_depth": (ctypes.c_int, [ctypes.c_int]),
    "zeta_search_last_ms": (ctypes.c_int, [ctypes.POINTER(ctypes.c_float)]),
    "zeta_search_last_table_ops": (ctypes.c_int, [_u64p, _u64p]),
    "zeta_genmoves_batch": (ctypes.c_int, [_u64p, _u8p, ctypes.c_int, ctypes.c_int, _u32p, _i32p]),
    "zeta_eval_batch": (ctypes.c_int, [_u64p, ctypes.c_int, _i32p]),
}

_lib: Optional[ctypes.CDLL] = None


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libzeta_cuda.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ZetaError(-3, f"{path} is missing: run __graft_entry__.build() (nvcc, sm_103a)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(rc: int) -> None:
    if rc != ZETA_OK:
        msg = load_library().zeta_last_error().decode(errors="replace")
        raise ZetaError(rc, msg)


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


# ---------------------------------------------------------------- lifecycle
def init(device: int = 0, tt1_mb: int = 0, tt2_mb: int = 0) -> None:
    _check(load_library().zeta_init(device, tt1_mb, tt2_mb))


def release() -> None:
    _check(load_library().zeta_release())


def device_info() -> dict:
    sms, ma, mi = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    hbm = ctypes.c_uint64()
    _check(load_library().zeta_device_info(ctypes.byref(sms), ctypes.byref(ma), ctypes.byref(mi), ctypes.byref(hbm)))
    return {"sms": sms.value, "cc": (ma.value, mi.value), "hbm_bytes": hbm.value}


# ---------------------------------------------------------------- perft
def perft(board: np.ndarray, stm: int, depth: int) -> int:
    b = np.ascontiguousarray(board, dtype=np.uint64).reshape(7)
    out = ctypes.c_uint64()
    _check(load_library().zeta_perft(_ptr(b, _u64p), int(stm), int(depth), ctypes.byref(out)))
    return out.value


def perft_batch(boards: np.ndarray, stm: np.ndarray, depth: np.ndarray) -> np.ndarray:
    b = np.ascontiguousarray(boards, dtype=np.uint64).reshape(-1, 7)
    s = np.ascontiguousarray(stm, dtype=np.uint8)
    d = np.ascontiguousarray(depth, dtype=np.uint8)
    n = b.shape[0]
    if s.shape != (n,) or d.shape != (n,):
        raise ValueError("stm and depth need one entry per board")
    out = np.zeros(n, dtype=np.uint64)
    _check(load_library().zeta_perft_batch(_ptr(b, _u64p), _ptr(s, _u8p), _ptr(d, _u8p), n, _ptr(out, _u64p)))
    return out


def perft_batch_device(d_boards: int, d_stm: int, d_depth: int, n: int, d_leaves: int, stream: int = 0) -> None:
    """Device pointers (e.g. torch ``data_ptr()``); ``stream`` a cudaStream_t handle."""
    _check(load_library().zeta_perft_batch_device(d_boards, d_stm, d_depth, n, d_leaves, stream))


def perft_configure(threads_per_block: int = 128, blocks_per_sm: int = 0, min_tasks: int = 0, task_depth: int = 3,
                    use_graph: bool = True) -> None:
    cfg = PerftConfig(threads_per_block, blocks_per_sm, min_tasks, task_depth, int(use_graph))
    _check(load_library().zeta_perft_configure(ctypes.byref(cfg)))


def perft_config() -> dict:
    cfg = PerftConfig()
    _check(load_library().zeta_perft_get_config(ctypes.byref(cfg)))
    return {f: getattr(cfg, f) for f, _ in PerftConfig._fields_}


def perft_set_promotions(all_pieces: bool) -> None:
    """Promotion rule of every perft entry: False (default) queen only, as
    the reference; True queen, rook, bishop or knight."""
    _check(load_library().zeta_perft_set_promotions(1 if all_pieces else 0))


def perft_get_promotions() -> bool:
    return load_library().zeta_perft_get_promotions() == 1


def perft_stats() -> dict:
    st = PerftStats()
    _check(load_library().zeta_perft_last_stats(ctypes.byref(st)))
    return {f: getattr(st, f) for f, _ in PerftStats._fields_}


# ---------------------------------------------------------------- positions / movegen
def make_positions(seed: int, n: int, min_plies: int, max_plies: int, min_pieces: int = 0, min_depth: int = 0,
                   max_depth: int = 0):
    boards = np.zeros((n, 7), dtype=np.uint64)
    stm = np.zeros(n, dtype=np.uint8)
    depth = np.zeros(n, dtype=np.uint8)
    _check(load_library().zeta_make_positions(seed & (2**64 - 1), n, min_plies, max_plies, min_pieces, min_depth,
                                              max_depth, _ptr(boards, _u64p), _ptr(stm, _u8p), _ptr(depth, _u8p)))
    return boards, stm, depth


def search_batch(boards: np.ndarray, stm: np.ndarray, depth: int, workers: int = 1):
    """Fixed-depth pure alpha-beta: (scores, best moves, nodes) per position."""
    b = np.ascontiguousarray(boards, dtype=np.uint64).reshape(-1, 7)
    s = np.ascontiguousarray(stm, dtype=np.uint8)
    n = b.shape[0]
    scores = np.zeros(n, dtype=np.int32)
    moves = np.zeros(n, dtype=np.uint32)
    nodes = np.zeros(n, dtype=np.uint64)
    _check(load_library().zeta_search_batch(_ptr(b, _u64p), _ptr(s, _u8p), n, depth, workers, _ptr(scores, _i32p),
                                            _ptr(moves, _u32p), _ptr(nodes, _u64p)))
    return scores, moves, nodes


def search_batch_device(d_boards: int, d_stm: int, n: int, depth: int, workers: int, d_scores: int, d_moves: int,
                        d_nodes: int, stream: int = 0) -> None:
    _check(load_library().zeta_search_batch_device(d_boards, d_stm, n, depth, workers, d_scores, d_moves, d_nodes,
                                                   stream or None))


def search_set_helpers(max_workers_per_position: int) -> None:
    _check(load_library().zeta_search_set_helpers(max_workers_per_position))


def engine_set_helper_depth(every: int) -> None:
    """Full engine, lazy SMP: every `every`-th helper one ply deeper (0 = off)."""
    _check(load_library().zeta_engine_set_helper_depth(int(every)))


def search_set_launch_form(form: int) -> None:
    """Search kernels' launch form: 0 automatic, 1 dense (32 workers per warp), 2 sparse (one per
    warp), 3 warp-cooperative (pure search: one worker per warp, the lanes score the last ply)."""
    _check(load_library().zeta_search_set_launch_form(form))


def gemm_configure(ctas_per_sm: int) -> None:
    """0 automatic (persistent), 1 / 2 per-tile kernel with its ring for 1 / 2 CTAs per SM, 3 persistent."""
    _check(load_library().zeta_gemm_configure(ctas_per_sm))


def gemm_tc(d_a: int, d_b: int, d_c: int, m: int, n: int, k: int, fp8: bool = False, stream: int = 0) -> None:
    """C[m x n] fp32 = A[m x k] . B[n x k]^T on the tcgen05 tensor cores (device pointers)."""
    _check(load_library().zeta_gemm_tc(d_a, d_b, d_c, m, n, k, int(fp8), stream or None))


_f32p = ctypes.POINTER(ctypes.c_float)

# layout of the network's flat FP32 parameter vector
MLP_SHAPES = [("W1", (512, 768)), ("b1", (512,)), ("W2", (256, 512)), ("b2", (256,)), ("W3", (128, 256)),
              ("b3", (128,)), ("Ef", (64, 64)), ("Et", (64, 64))]


def mlp_init(seed: int = 1) -> None:
    _check(load_library().zeta_mlp_init(seed))


def mlp_get_params() -> np.ndarray:
    p = np.zeros(load_library().zeta_mlp_param_count(), dtype=np.float32)
    _check(load_library().zeta_mlp_get_params(_ptr(p, _f32p)))
    return p


def mlp_set_params(p: np.ndarray) -> None:
    p = np.ascontiguousarray(p, dtype=np.float32)
    _check(load_library().zeta_mlp_set_params(_ptr(p, _f32p)))


def mlp_unflatten(p: np.ndarray) -> dict:
    out, off = {}, 0
    for name, shape in MLP_SHAPES:
        n = int(np.prod(shape))
        out[name] = p[off:off + n].reshape(shape)
        off += n
    return out


def mlp_grads(boards, stm, targets):
    b = np.ascontiguousarray(boards, dtype=np.uint64).reshape(-1, 7)
    s = np.ascontiguousarray(stm, dtype=np.uint8)
    t = np.ascontiguousarray(targets, dtype=np.uint32)
    g = np.zeros(load_library().zeta_mlp_param_count(), dtype=np.float32)
    loss = ctypes.c_float()
    _check(load_library().zeta_mlp_grads(_ptr(b, _u64p), _ptr(s, _u8p), _ptr(t, _u32p), b.shape[0], _ptr(g, _f32p),
                                         ctypes.byref(loss)))
    return g, loss.value


def mlp_train(boards, stm, targets, epochs: int = 1, batch: int = 4096, lr: float = 1e-3):
    b = np.ascontiguousarray(boards, dtype=np.uint64).reshape(-1, 7)
    s = np.ascontiguousarray(stm, dtype=np.uint8)
    t = np.ascontiguousarray(targets, dtype=np.uint32)
    loss = np.zeros(epochs, dtype=np.float32)
    acc = np.zeros(epochs, dtype=np.float32)
    _check(load_library().zeta_mlp_train(_ptr(b, _u64p), _ptr(s, _u8p), _ptr(t, _u32p), b.shape[0], epochs, batch,
                                         lr, _ptr(loss, _f32p), _ptr(acc, _f32p)))
    return loss, acc


def mlp_scores(boards, stm, fp8: bool = False):
    """(scores n x 218, counts n, best index n) of every legal move, in the
    engine's move-generation order."""
    b = np.ascontiguousarray(boards, dtype=np.uint64).reshape(-1, 7)
    s = np.ascontiguousarray(stm, dtype=np.uint8)
    n = b.shape[0]
    sc = np.zeros((n, 218), dtype=np.float32)
    nm = np.zeros(n, dtype=np.uint8)
    best = np.zeros(n, dtype=np.int32)
    _check(load_library().zeta_mlp_scores(_ptr(b, _u64p), _ptr(s, _u8p), n, int(fp8), _ptr(sc, _f32p), _ptr(nm, _u8p),
                                          _ptr(best, _i32p)))
    return sc, nm, best


def search_id(boards, stm, depth: int, workers: int = 32, ordering: int = 0):
    """Iterative deepening to `depth`; ordering 0 hand-written, 1 network
    (BF16), 2 network (FP8).  Returns (scores, moves, nodes, ms_total,
    ms_search, ms_network)."""
    b = np.ascontiguousarray(boards, dtype=np.uint64).reshape(-1, 7)
    s = np.ascontiguousarray(stm, dtype=np.uint8)
    n = b.shape[0]
    scores = np.zeros(n, dtype=np.int32)
    moves = np.zeros(n, dtype=np.uint32)
    nodes = np.zeros(n, dtype=np.uint64)
    t = [ctypes.c_float() for _ in range(3)]
    _check(load_library().zeta_search_id(_ptr(b, _u64p), _ptr(s, _u8p), n, depth, workers, ordering,
                                         _ptr(scores, _i32p), _ptr(moves, _u32p), _ptr(nodes, _u64p),
                                         ctypes.byref(t[0]), ctypes.byref(t[1]), ctypes.byref(t[2])))
    return scores, moves, nodes, t[0].value, t[1].value, t[2].value


def engine_search(board, stm: int, depth: int, workers: int = 1, ply_init: int = 0, hash_history=None,
                  max_nodes: int = (1 << 63)):
    """One full-engine search launch: (pv uint32[64], counters uint64[workers, 64])."""
    b = np.ascontiguousarray(board, dtype=np.uint64).reshape(7)
    h = None if hash_history is None else np.ascontiguousarray(hash_history, dtype=np.uint64).reshape(1024)
    pv = np.zeros(64, dtype=np.uint32)
    cnt = np.zeros((workers, 64), dtype=np.uint64)
    _check(load_library().zeta_engine_search(_ptr(b, _u64p), int(stm), depth, ply_init,
                                             _ptr(h, _u64p) if h is not None else None, max_nodes, workers,
                                             _ptr(pv, _u32p), _ptr(cnt, _u64p)))
    return pv, cnt


def engine_batch(boards, stm, depth: int, workers: int = 1, max_nodes: int = (1 << 63), with_pv: bool = False):
    """Full-engine search of n positions in one launch: (scores, best moves,
    nodes[, pvs n x 64])."""
    b = np.ascontiguousarray(boards, dtype=np.uint64).reshape(-1, 7)
    s = np.ascontiguousarray(stm, dtype=np.uint8)
    n = b.shape[0]
    scores = np.zeros(n, dtype=np.int32)
    moves = np.zeros(n, dtype=np.uint32)
    nodes = np.zeros(n, dtype=np.uint64)
    pvs = np.zeros((n, 64), dtype=np.uint32) if with_pv else None
    _check(load_library().zeta_engine_batch(_ptr(b, _u64p), _ptr(s, _u8p), n, depth, workers, max_nodes,
                                            _ptr(scores, _i32p), _ptr(moves, _u32p), _ptr(nodes, _u64p),
                                            _ptr(pvs, _u32p) if with_pv else None))
    return (scores, moves, nodes, pvs) if with_pv else (scores, moves, nodes)


def engine_id(boards, stm, depth: int, workers: int = 1, ordering: int = 0, max_nodes: int = 0):
    """Iterative deepening of n positions with the full engine: (scores,
    best moves, nodes, depth reached, ms_total, ms_search, ms_network)."""
    b = np.ascontiguousarray(boards, dtype=np.uint64).reshape(-1, 7)
    s = np.ascontiguousarray(stm, dtype=np.uint8)
    n = b.shape[0]
    scores = np.zeros(n, dtype=np.int32)
    moves = np.zeros(n, dtype=np.uint32)
    nodes = np.zeros(n, dtype=np.uint64)
    dd = np.zeros(n, dtype=np.uint8)
    t = [ctypes.c_float() for _ in range(3)]
    _check(load_library().zeta_engine_id(_ptr(b, _u64p), _ptr(s, _u8p), n, depth, workers, max_nodes, ordering,
                                         _ptr(scores, _i32p), _ptr(moves, _u32p), _ptr(nodes, _u64p), _ptr(dd, _u8p),
                                         ctypes.byref(t[0]), ctypes.byref(t[1]), ctypes.byref(t[2])))
    return scores, moves, nodes, dd, t[0].value, t[1].value, t[2].value


def search_set_learned_order(top: int = 12, quiet_only: bool = True) -> None:
    _check(load_library().zeta_search_set_learned_order(top, int(quiet_only)))


def tt_clear() -> None:
    _check(load_library().zeta_tt_clear())


def search_last_ms() -> float:
    t = ctypes.c_float()
    _check(load_library().zeta_search_last_ms(ctypes.byref(t)))
    return t.value


def search_last_table_ops() -> tuple[int, int]:
    """(probes, stores) of the transposition table in the last batched search."""
    a, b = ctypes.c_uint64(), ctypes.c_uint64()
    _check(load_library().zeta_search_last_table_ops(ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


def int_peak_tops() -> float:
    """Measured int32 ALU throughput (Tops/s) of the initialised device."""
    t = ctypes.c_double()
    _check(load_library().zeta_int_peak(ctypes.byref(t)))
    return t.value


def genmoves_batch(boards: np.ndarray, stm: np.ndarray, qs: bool = False, generator: int = 0,
                   all_promotions: bool = False):
    """Legal moves on the device; generator 0 the perft generator, 1 the
    search kernels', 2 the warp-cooperative search's; all_promotions (perft
    generator only) adds the rook, bishop and knight promotions."""
    b = np.ascontiguousarray(boards, dtype=np.uint64).reshape(-1, 7)
    s = np.ascontiguousarray(stm, dtype=np.uint8)
    n = b.shape[0]
    moves = np.zeros((n, 256), dtype=np.uint32)
    counts = np.zeros(n, dtype=np.int32)
    flags = int(qs) | (generator << 1) | (8 if all_promotions else 0)
    _check(load_library().zeta_genmoves_batch(_ptr(b, _u64p), _ptr(s, _u8p), n, flags, _ptr(moves, _u32p),
                                              _ptr(counts, _i32p)))
    return [moves[i, : counts[i]].copy() for i in range(n)]


def eval_batch(boards: np.ndarray) -> np.ndarray:
    """Static evaluation (white's view) of n boards on the device."""
    b = np.ascontiguousarray(boards, dtype=np.uint64).reshape(-1, 7)
    out = np.zeros(b.shape[0], dtype=np.int32)
    _check(load_library().zeta_eval_batch(_ptr(b, _u64p), b.shape[0], _ptr(out, _i32p)))
    return out


# workload definitions of the benchmark configurations (seeded, synthetic)
SEED_BASE = 0x5A17A0000000001
WORKLOADS = {
    # batched perft: 4096 playouts of 10-60 plies, depth 3-5
    "perft_batch": dict(seed=SEED_BASE + 2, n=4096, min_plies=10, max_plies=60, min_pieces=0, min_depth=3,
                        max_depth=5),
    # batched search: 1024 playouts of 20-40 plies with >= 20 pieces
    "search_batch": dict(seed=SEED_BASE + 3, n=1024, min_plies=20, max_plies=40, min_pieces=20, min_depth=7,
                         max_depth=7),
    # full engine: 256 playouts of 20-40 plies with >= 20 pieces
    "engine": dict(seed=SEED_BASE + 5, n=256, min_plies=20, max_plies=40, min_pieces=20, min_depth=12,
                   max_depth=12),
}

# the initial position as setboard leaves it (src/io.c:335-531), white to move
STARTPOS = np.array([0xFFFF000000000000, 0x91FF00000000FF91, 0x5A0000000000005A, 0xAD000000000000AD,
                     0x6EFFFFFFFFFFFF6E, 0x18892007F9451009, 0], dtype=np.uint64)
