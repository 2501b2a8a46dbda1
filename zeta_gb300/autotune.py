"""Autotuners of the batched kernels (the full engine's single-position
search is tuned by the host's --guessconfig, zeta_gb300/host/cudarun.c).

Replace the reference's --guessconfigx search (src/clconfig.c:33-1058,
src/bench.c:109-160), which doubled the number of workers while nodes/s
kept improving by 1.68x.  Here every setting is timed on the benchmark
workload itself (device-resident batch, CUDA-event timing), its results are
checked against the first setting's, and the fastest is recorded:

* perft: every compiled kernel variant (threads per block x register cap)
  x task depth -> ``zeta_gb300/perft_tuned.json``, applied by
  ``load_tuned()``;
* batched pure search: launch form x ABDADA workers per position x helper
  cap, then the transposition-table size of the best -> 
  ``zeta_gb300/search_tuned.json``, read by ``load_search_tuned()``.

    python -m zeta_gb300.autotune [perft|search] [--n N] [--reps R]
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TUNED = os.path.join(HERE, "perft_tuned.json")

# (threads_per_block, blocks_per_sm) pairs compiled into libzeta_cuda.so
VARIANTS = [(64, 0), (64, 8), (64, 12), (128, 0), (128, 4), (128, 6), (256, 0), (256, 3), (512, 0)]
TASK_DEPTHS = (3, 4)


def load_tuned(z=None) -> dict | None:
    """Apply the tuned perft configuration, if one was recorded."""
    if not os.path.exists(TUNED):
        return None
    import zeta_gb300 as zz
    z = z or zz
    best = json.load(open(TUNED))["best"]
    z.perft_configure(threads_per_block=best["threads_per_block"], blocks_per_sm=best["blocks_per_sm"],
                      min_tasks=best.get("min_tasks", 0), task_depth=best["task_depth"], use_graph=True)
    return best


def tune(n: int = 0, reps: int = 3, write: bool = True) -> dict:
    import torch
    import zeta_gb300 as z
    z.init(0, 0, 0)
    w = dict(z.WORKLOADS["perft_batch"])
    boards, stm, depth = z.make_positions(w["seed"], n or w["n"], w["min_plies"], w["max_plies"], w["min_pieces"],
                                          w["min_depth"], w["max_depth"])
    n = len(depth)
    dev = torch.device("cuda", 0)
    d_b = torch.from_numpy(boards.view(np.int64)).to(dev)
    d_s = torch.from_numpy(stm).to(dev)
    d_d = torch.from_numpy(depth).to(dev)
    d_l = torch.zeros(n, dtype=torch.int64, device=dev)
    stream = torch.cuda.Stream(dev)
    results, ref = [], None
    for tpb, bps in VARIANTS:
        for td in TASK_DEPTHS:
            z.perft_configure(threads_per_block=tpb, blocks_per_sm=bps, min_tasks=0, task_depth=td, use_graph=True)
            try:
                z.perft_batch_device(d_b.data_ptr(), d_s.data_ptr(), d_d.data_ptr(), n, d_l.data_ptr(),
                                     stream.cuda_stream)
            except z.ZetaError as e:
                results.append({"threads_per_block": tpb, "blocks_per_sm": bps, "task_depth": td, "error": str(e)})
                continue
            counts = d_l.cpu().numpy().view(np.uint64).copy()
            if ref is None:
                ref = counts
            if not np.array_equal(counts, ref):
                raise SystemExit(f"counts differ under {tpb}x{bps} depth {td}")
            ms = []
            for _ in range(reps):
                z.perft_batch_device(d_b.data_ptr(), d_s.data_ptr(), d_d.data_ptr(), n, d_l.data_ptr(),
                                     stream.cuda_stream)
                ms.append(z.perft_stats()["kernel_ms"])
            st = z.perft_stats()
            best_ms = min(ms)
            results.append({"threads_per_block": tpb, "blocks_per_sm": bps, "task_depth": td, "kernel_ms": best_ms,
                            "leaves_per_s": float(ref.sum()) / (best_ms / 1e3), "tasks": st["tasks"],
                            "steals": st["steals"]})
            print(json.dumps(results[-1]), flush=True)
    ok = [r for r in results if "kernel_ms" in r]
    best = max(ok, key=lambda r: r["leaves_per_s"])
    out = {"best": best, "all": results, "workload": f"perft_batch n={n}", "when": time.strftime("%Y-%m-%d %H:%M:%S"),
           "device": z.device_info()}
    if write:
        json.dump(out, open(TUNED, "w"), indent=1)
    z.release()
    return out


SEARCH_TUNED = os.path.join(HERE, "search_tuned.json")
# the setting used when none was recorded: warp-cooperative, 2 workers per
# position, helpers up to 64 per position, 1 GiB table
SEARCH_DEFAULT = {"form": 3, "workers": 2, "helpers": 64, "tt_mb": 1024}
# (launch form, workers per position, helper cap): 1 dense, 3 warp-cooperative
SEARCH_GRID = [(1, 32, 128), (3, 1, 16), (3, 1, 32), (3, 2, 16), (3, 2, 32), (3, 2, 64), (3, 3, 32), (3, 3, 64)]
SEARCH_TT_MB = (256, 1024, 4096)


def load_search_tuned() -> dict:
    """The recorded batched-search setting, else SEARCH_DEFAULT."""
    if os.path.exists(SEARCH_TUNED):
        return dict(SEARCH_DEFAULT, **json.load(open(SEARCH_TUNED))["best"])
    return dict(SEARCH_DEFAULT)


def tune_search(n: int = 0, depth: int = 7, reps: int = 2, write: bool = True) -> dict:
    """Every (form, workers, helper cap) of SEARCH_GRID on the batched-search
    workload at a 1 GiB table, then the best one at each table size of
    SEARCH_TT_MB; root scores must agree across all settings."""
    import torch
    import zeta_gb300 as z
    w = dict(z.WORKLOADS["search_batch"])
    z.init(0, 1024, 0)
    boards, stm, _ = z.make_positions(w["seed"], n or w["n"], w["min_plies"], w["max_plies"], w["min_pieces"], 0, 0)
    n = len(stm)
    dev = torch.device("cuda", 0)
    d_b = torch.from_numpy(boards.view(np.int64)).to(dev)
    d_s = torch.from_numpy(stm).to(dev)
    d_sc = torch.zeros(n, dtype=torch.int32, device=dev)
    d_mv = torch.zeros(n, dtype=torch.int32, device=dev)
    d_nd = torch.zeros(n, dtype=torch.int64, device=dev)
    stream = torch.cuda.Stream(dev)
    results, ref = [], None

    def measure(form, workers, helpers, tt_mb):
        nonlocal ref
        z.search_set_launch_form(form)
        z.search_set_helpers(helpers)
        ms = []
        for k in range(reps + 1):  # one warm-up
            z.tt_clear()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            z.search_batch_device(d_b.data_ptr(), d_s.data_ptr(), n, depth, workers, d_sc.data_ptr(),
                                  d_mv.data_ptr(), d_nd.data_ptr(), stream.cuda_stream)
            if k:
                ms.append((time.perf_counter() - t0) * 1e3)
        sc = d_sc.cpu().numpy().copy()
        if ref is None:
            ref = sc
        if not np.array_equal(sc, ref):
            raise SystemExit(f"root scores differ under form {form}, {workers} workers, cap {helpers}")
        r = {"form": form, "workers": workers, "helpers": helpers, "tt_mb": tt_mb, "ms": min(ms),
             "positions_per_s": n / (min(ms) / 1e3), "nodes": int(d_nd.sum().item())}
        results.append(r)
        print(json.dumps(r), flush=True)
        return r

    try:
        for form, workers, helpers in SEARCH_GRID:
            measure(form, workers, helpers, 1024)
        best = max(results, key=lambda r: r["positions_per_s"])
        for tt_mb in SEARCH_TT_MB:
            if tt_mb == 1024:
                continue
            z.release()
            z.init(0, tt_mb, 0)
            measure(best["form"], best["workers"], best["helpers"], tt_mb)
        best = max(results, key=lambda r: r["positions_per_s"])
    finally:
        z.search_set_launch_form(0)
        z.search_set_helpers(0)
        z.release()
    out = {"best": {k: best[k] for k in ("form", "workers", "helpers", "tt_mb")}, "best_positions_per_s":
           best["positions_per_s"], "all": results, "workload": f"search_batch n={n} depth {depth}",
           "when": time.strftime("%Y-%m-%d %H:%M:%S")}
    if write:
        json.dump(out, open(SEARCH_TUNED, "w"), indent=1)
    return out


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("what", nargs="?", choices=["perft", "search"], default="perft")
    ap.add_argument("--n", type=int, default=0)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    r = tune(a.n, a.reps) if a.what == "perft" else tune_search(a.n, reps=a.reps)
    print("best:", json.dumps(r["best"]))
