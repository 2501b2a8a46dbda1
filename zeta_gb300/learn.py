"""Learned move ordering: data, training and the A/B test.

1. Data: seeded random-playout positions labelled with the best move of
   the plain fixed-depth search on the GPU (the engine's own search is the
   teacher).
2. Training: the tensor-core network (zeta_mlp_train: BF16 forward and
   backward GEMMs, Adam in FP32).
3. A/B: iterative deepening to a depth with the hand-written ordering and
   with the network's ordering (BF16 or FP8) on the same positions; the
   root scores must be identical, nodes and time-to-depth are compared.

    python -m zeta_gb300.learn train [--n 524288] [--label-depth 6] [--epochs 20]
    python -m zeta_gb300.learn ab [--n 1024] [--depth 8]
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MODEL = os.path.join(HERE, "models", "ordering_params.npy")
TRAIN_SEED = 0x5A17A0000000004   # disjoint from the evaluation workloads' seeds


def make_dataset(z, n: int, label_depth: int, seed: int = TRAIN_SEED, workers: int = 2, helpers: int = 64,
                 chunk: int = 1024):
    """n positions (10-60 random plies) and the plain search's best move at
    label_depth, `chunk` positions per launch with `workers` ABDADA workers
    each and finished workers helping up to `helpers` per position (one warp
    per worker: the warp-cooperative form, the fastest measured)."""
    boards, stm, _ = z.make_positions(seed, n, 10, 60, 0, 0, 0)
    best = np.zeros(n, dtype=np.uint32)
    z.search_set_helpers(helpers)
    try:
        for off in range(0, n, chunk):
            z.tt_clear()
            _, mv, _ = z.search_batch(boards[off:off + chunk], stm[off:off + chunk], label_depth, workers)
            best[off:off + chunk] = mv
    finally:
        z.search_set_helpers(0)
    return boards, stm, best


def train(z, boards, stm, best, epochs: int = 10, batch: int = 4096, lr: float = 1e-3, seed: int = 1):
    z.mlp_init(seed)
    return z.mlp_train(boards, stm, best, epochs=epochs, batch=batch, lr=lr)


def top1(z, boards, stm, best, fp8: bool = False) -> float:
    """Share of positions whose highest-scored legal move is the label."""
    _, _, arg = z.mlp_scores(boards, stm, fp8=fp8)
    hit = 0
    mv = z.genmoves_batch(boards, stm)
    for i in range(len(best)):
        if 0 <= arg[i] < len(mv[i]) and int(mv[i][arg[i]]) == int(best[i]):
            hit += 1
    return hit / max(1, len(best))


def save(z, path: str = MODEL):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.save(path, z.mlp_get_params())


def load(z, path: str = MODEL) -> bool:
    if not os.path.exists(path):
        return False
    z.mlp_init(1)
    z.mlp_set_params(np.load(path))
    return True


def ab_test(z, boards, stm, depth: int, workers: int = 32, orderings=((0, 12, 1), (1, 12, 1), (2, 12, 1))):
    """Iterative deepening to `depth` under each (ordering, top, quiet_only)
    from a cleared table each time.  Returns per-case scores, nodes and
    times, keyed "plain" or "bf16/fp8-top<k>[-quiet]"."""
    out = {}
    for o, top, quiet in orderings:
        z.search_set_learned_order(top, bool(quiet))
        z.tt_clear()
        sc, mv, nodes, ms, ms_s, ms_n = z.search_id(boards, stm, depth, workers, o)
        key = "plain" if o == 0 else f"{'bf16' if o == 1 else 'fp8'}-top{top}{'-quiet' if quiet else ''}"
        out[key] = {"scores": sc, "moves": mv, "nodes": int(nodes.sum()), "ms_total": ms, "ms_search": ms_s,
                    "ms_network": ms_n}
    z.search_set_learned_order(12, True)
    return out


def main():
    import zeta_gb300 as z
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train", "ab"])
    ap.add_argument("--n", type=int, default=0)
    ap.add_argument("--label-depth", type=int, default=6)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--depth", type=int, default=8)
    ap.add_argument("--workers", type=int, default=32)
    ap.add_argument("--out", default="")
    ap.add_argument("--cases", default="0:12:1,1:12:1,2:12:1",
                    help="comma-separated ordering:top:quiet_only cases of the A/B")
    a = ap.parse_args()
    z.init(0, 1024, 0)
    if a.cmd == "train":
        n = a.n or 524288
        t0 = time.time()
        boards, stm, best = make_dataset(z, n, a.label_depth)
        t1 = time.time()
        hold = max(1024, n // 16)   # held-out tail
        loss, acc = train(z, boards[:-hold], stm[:-hold], best[:-hold], epochs=a.epochs)
        t2 = time.time()
        save(z, a.out or MODEL)
        print(json.dumps({"positions": n, "label_depth": a.label_depth, "label_s": round(t1 - t0, 2),
                          "train_s": round(t2 - t1, 2), "loss": [round(float(x), 4) for x in loss],
                          "top1": [round(float(x), 4) for x in acc],
                          "heldout_top1_bf16": round(top1(z, boards[-hold:], stm[-hold:], best[-hold:]), 4),
                          "heldout_top1_fp8": round(top1(z, boards[-hold:], stm[-hold:], best[-hold:], True), 4)}),
              flush=True)
    else:
        if not load(z, a.out or MODEL):
            raise SystemExit("no trained model: run `python -m zeta_gb300.learn train` first")
        w = z.WORKLOADS["search_batch"]
        n = a.n or w["n"]
        boards, stm, _ = z.make_positions(w["seed"], n, w["min_plies"], w["max_plies"], w["min_pieces"], 0, 0)
        cases = [tuple(int(x) for x in c.split(":")) for c in a.cases.split(",")]
        r = ab_test(z, boards, stm, a.depth, a.workers, cases)
        ref = next(iter(r.values()))["scores"]
        same = all(np.array_equal(ref, r[o]["scores"]) for o in r)
        print(json.dumps({"depth": a.depth, "positions": n, "scores_identical": bool(same),
                          **{o: {k: v for k, v in r[o].items() if k not in ("scores", "moves")} for o in r}}),
              flush=True)
    z.release()


if __name__ == "__main__":
    main()
