"""Autotuner of the perft launch (block size, register cap, task depth).

Replaces the reference's --guessconfigx search (src/clconfig.c:33-1058,
src/bench.c:109-160), which doubled the number of workers while nodes/s
kept improving by 1.68x.  Here every compiled kernel variant is timed on
the benchmark workload itself (device-resident batch, CUDA-event timing of
the work-stealing kernel), its leaf counts are checked against the first
configuration's, and the fastest configuration is written to
``zeta_gb300/perft_tuned.json``; ``load_tuned()`` applies it.

    python -m zeta_gb300.autotune [--n 4096] [--reps 3]
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


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=0)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    r = tune(a.n, a.reps)
    print("best:", json.dumps(r["best"]))
