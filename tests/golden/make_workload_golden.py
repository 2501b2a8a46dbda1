"""Golden fixtures for the benchmark workloads at their configured depths.

    python tests/golden/make_workload_golden.py [--procs 8] [--perft] [--search] [--promotions]

perft_workload.json
    The batched-perft workload (4096 seeded playouts of 10-60 plies, depth
    drawn from 3-5; seed 0x5A17A0000000001 + 2): the SHA-256 of the
    positions' bytes, the oracle's leaf count of every position at its drawn
    depth, and, for 16 of them (the first 12 of depth 4 and the first 4 of
    depth 5), the count of the reference's own perft kernel (oracle/_ref,
    unmodified zetaperft.cl on host cores), which must equal the oracle's.
search_workload.json
    The batched-search workload (1024 playouts of 20-40 plies with at least
    20 pieces; seed 0x5A17A0000000001 + 3): the oracle's plain alpha-beta
    root score at depth 7 (the configured depth) of the first 128 positions,
    with the oracle's best move and visited nodes.  The value comes from
    zo_alphabeta_ordered, which is full-window alpha-beta with reordered
    moves; the script checks it against zo_alphabeta on every position at
    depth 4 first.

perft_promotions.json
    Perft with promotion to any of the four pieces (the reference promotes
    to a queen only, so no reference output exists for it): the oracle's
    count (zo_perft_ex) of every batched-perft workload position at its
    drawn depth, the positions whose count differs from the queen-only one,
    and five hand-made positions (push, capture and check-blocking
    promotions, a promotion that cannot answer a check, a pinned pawn) at
    depths 1-5 under both rules.  The independent mailbox generator
    (tests/mailbox_gen.py) recomputes every hand-made count up to depth 4 and
    the differing workload positions of depth 3, both rules, and must
    agree.

The positions are made by the oracle's generator (zo_make_position), the
same bytes the device generator makes (checked by the GPU tests).  Work is
spread over host processes started with `spawn`.  Only the JSON files are
read at test time.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

SEED_BASE = 0x5A17A0000000001
PERFT = dict(seed=SEED_BASE + 2, n=4096, min_plies=10, max_plies=60, min_pieces=0, min_depth=3, max_depth=5)
SEARCH = dict(seed=SEED_BASE + 3, n=1024, min_plies=20, max_plies=40, min_pieces=20, min_depth=7, max_depth=7)
SEARCH_FIXTURE_POSITIONS = 128
SEARCH_DEPTH = 7


def positions_sha256(boards, stm, depth) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(boards, dtype="<u8").tobytes())
    h.update(np.ascontiguousarray(stm, dtype=np.uint8).tobytes())
    h.update(np.ascontiguousarray(depth, dtype=np.uint8).tobytes())
    return h.hexdigest()


def _make(w, n=None):
    import oracle_lib as ol
    return ol.make_positions(w["seed"], n or w["n"], min_plies=w["min_plies"], max_plies=w["max_plies"],
                             min_pieces=w["min_pieces"], min_depth=w["min_depth"], max_depth=w["max_depth"])


def _oracle_perft(args):
    import oracle_lib as ol
    board, stm, depth = args
    return int(ol.perft(np.array(board, dtype=np.uint64), stm, depth))


def _oracle_perft_all(args):
    import oracle_lib as ol
    board, stm, depth = args
    return int(ol.perft(np.array(board, dtype=np.uint64), stm, depth, all_promotions=True))


def _mailbox_perft(args):
    import mailbox_gen as mailbox
    board, stm, depth, all_promotions = args
    return int(mailbox.board_perft(board, stm, depth, all_promotions))


# hand-made positions with promotions: (FEN, what it exercises)
PROMOTION_FENS = [
    ("4k3/1P4P1/8/8/8/8/1p4p1/4K3 w - - 0 1", "pushes to the last rank, both sides"),
    ("r1n1k3/1P6/8/8/8/8/6p1/4K2R b K - 0 1", "captures onto the last rank, a castle right"),
    ("K6r/2P5/8/8/8/8/8/3k4 w - - 0 1", "a promotion that blocks a check"),
    ("3k4/2P5/8/8/8/8/8/K6r w - - 0 1", "in check: no promotion answers it"),
    ("8/8/8/8/8/k7/1p6/2B4K b - - 0 1", "a pinned pawn: capture along the pin only"),
]
PROMOTION_FEN_DEPTH = 5
MAILBOX_DEPTH = 4


def make_promotions(procs: int) -> dict:
    import oracle_lib as ol
    boards, stm, depth = _make(PERFT)
    queen = json.load(open(os.path.join(HERE, "perft_workload.json")))
    if queen["positions_sha256"] != positions_sha256(boards, stm, depth):
        raise AssertionError("perft_workload.json was made from other positions")
    t = time.time()
    jobs = [([int(x) for x in boards[i]], int(stm[i]), int(depth[i])) for i in range(len(depth))]
    with mp.get_context("spawn").Pool(procs) as pool:
        leaves = pool.map(_oracle_perft_all, jobs, chunksize=4)
        differ = [i for i in range(len(leaves)) if leaves[i] != queen["leaves"][i]]
        print(f"oracle, all promotions: {sum(leaves)} leaves in {time.time() - t:.0f}s; "
              f"{len(differ)} positions differ from queen-only", flush=True)
        # the mailbox generator on the differing positions of depth 3
        d3 = [i for i in differ if depth[i] == 3]
        mjobs = [(jobs[i][0], jobs[i][1], 3, ap) for i in d3 for ap in (False, True)]
        mres = pool.map(_mailbox_perft, mjobs, chunksize=1)
        for k, i in enumerate(d3):
            if (mres[2 * k], mres[2 * k + 1]) != (queen["leaves"][i], leaves[i]):
                raise AssertionError(f"mailbox {mres[2 * k:2 * k + 2]} != oracle at workload position {i}")
        special = []
        fjobs = []
        for fen, what in PROMOTION_FENS:
            b, s = ol.setboard(fen)
            row = {"fen": fen, "what": what, "queen_only": [], "all_promotions": []}
            for d in range(1, PROMOTION_FEN_DEPTH + 1):
                row["queen_only"].append(int(ol.perft(b, s, d)))
                row["all_promotions"].append(int(ol.perft(b, s, d, all_promotions=True)))
                if d <= MAILBOX_DEPTH:
                    fjobs += [([int(x) for x in b], s, d, False), ([int(x) for x in b], s, d, True)]
            special.append(row)
        fres = pool.map(_mailbox_perft, fjobs, chunksize=1)
    k = 0
    for row in special:
        for d in range(MAILBOX_DEPTH):
            if (fres[k], fres[k + 1]) != (row["queen_only"][d], row["all_promotions"][d]):
                raise AssertionError(f"mailbox {fres[k:k + 2]} != oracle for {row['fen']} at depth {d + 1}")
            k += 2
    print(f"mailbox: {len(d3)} workload positions of depth 3 and {len(special)} hand-made positions agree",
          flush=True)
    return {"workload": {k: (hex(v) if k == "seed" else v) for k, v in PERFT.items()},
            "positions_sha256": positions_sha256(boards, stm, depth),
            "leaves": leaves, "total_leaves": int(sum(leaves)), "differ_from_queen_only": differ,
            "mailbox_checked_workload": d3, "special": special, "mailbox_depth": MAILBOX_DEPTH,
            "source": "oracle/zeta_oracle.c zo_perft_ex (all four promotions), cross-checked by "
                      "tests/mailbox_gen.py"}


def _oracle_search(args):
    import oracle_lib as ol
    board, stm, depth = args
    b = np.array(board, dtype=np.uint64)
    v4, _, _ = ol.alphabeta(b, stm, 4)
    o4, _, _ = ol.alphabeta_ordered(b, stm, 4)
    if v4 != o4:
        raise AssertionError(f"ordered alpha-beta {o4} != alpha-beta {v4} at depth 4")
    v, m, nodes = ol.alphabeta_ordered(b, stm, depth)
    return int(v), int(m), int(nodes)


def _reference_perft(board, stm: int, depth: int, threads: int) -> int:
    """The reference kernel's count, fanned out over the grandchildren."""
    import oracle_lib as ol
    if depth <= 2:
        return ol.ref_perft(board, stm, depth)
    kids, kstm = [], []
    for m in ol.genmoves(board, stm):
        c = ol.play(board, stm, m, True)
        for m2 in ol.genmoves(c, 1 - stm):
            kids.append(ol.play(c, 1 - stm, m2, True))
            kstm.append(stm)
    if not kids:
        return 0
    out = ol.ref_perft_batch(np.array(kids), np.array(kstm), np.full(len(kids), depth - 2), threads)
    return int(out.sum())


def make_perft(procs: int) -> dict:
    import oracle_lib as ol
    boards, stm, depth = _make(PERFT)
    t = time.time()
    with mp.get_context("spawn").Pool(procs) as pool:
        jobs = [([int(x) for x in boards[i]], int(stm[i]), int(depth[i])) for i in range(len(depth))]
        leaves = pool.map(_oracle_perft, jobs, chunksize=4)
    print(f"oracle: {sum(leaves)} leaves over {len(leaves)} positions in {time.time() - t:.0f}s", flush=True)
    subset = []
    if ol.reference() is not None:
        pick = [i for i in range(len(depth)) if depth[i] == 4][:12] + [i for i in range(len(depth)) if depth[i] == 5][:4]
        for i in pick:
            t = time.time()
            r = _reference_perft(boards[i], int(stm[i]), int(depth[i]), procs)
            print(f"reference: position {i} depth {depth[i]}: {r} ({time.time() - t:.0f}s)", flush=True)
            if r != leaves[i]:
                raise AssertionError(f"reference {r} != oracle {leaves[i]} at position {i}")
            subset.append({"index": i, "depth": int(depth[i]), "leaves": r})
    return {"workload": {k: (hex(v) if k == "seed" else v) for k, v in PERFT.items()},
            "positions_sha256": positions_sha256(boards, stm, depth),
            "depth_histogram": {str(d): int((depth == d).sum()) for d in (3, 4, 5)},
            "leaves": leaves, "total_leaves": int(sum(leaves)),
            "source": "oracle/zeta_oracle.c zo_perft (restatement of src/zetaperft.cl:801-1477)",
            "reference_subset": subset,
            "reference_source": "unmodified src/zetaperft.cl on host cores (oracle/_ref)"}


def make_search(procs: int) -> dict:
    boards, stm, _ = _make(SEARCH, SEARCH_FIXTURE_POSITIONS)
    full_b, full_s, full_d = _make(SEARCH)
    t = time.time()
    with mp.get_context("spawn").Pool(procs) as pool:
        jobs = [([int(x) for x in boards[i]], int(stm[i]), SEARCH_DEPTH) for i in range(len(stm))]
        res = pool.map(_oracle_search, jobs, chunksize=1)
    print(f"oracle search: {len(res)} positions at depth {SEARCH_DEPTH} in {time.time() - t:.0f}s", flush=True)
    return {"workload": {k: (hex(v) if k == "seed" else v) for k, v in SEARCH.items()},
            "positions_sha256": positions_sha256(full_b, full_s, full_d),
            "depth": SEARCH_DEPTH, "positions": SEARCH_FIXTURE_POSITIONS,
            "scores": [r[0] for r in res], "bestmoves": [r[1] for r in res], "oracle_nodes": [r[2] for r in res],
            "source": "oracle/zeta_oracle.c zo_alphabeta_ordered (plain alpha-beta value, no TT, "
                      "checked against zo_alphabeta at depth 4)"}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--procs", type=int, default=os.cpu_count() or 8)
    ap.add_argument("--perft", action="store_true")
    ap.add_argument("--search", action="store_true")
    ap.add_argument("--promotions", action="store_true")
    a = ap.parse_args()
    if not (a.perft or a.search or a.promotions):
        a.perft = a.search = a.promotions = True
    if a.search:
        json.dump(make_search(a.procs), open(os.path.join(HERE, "search_workload.json"), "w"), indent=0)
    if a.perft:
        json.dump(make_perft(a.procs), open(os.path.join(HERE, "perft_workload.json"), "w"), indent=0)
    if a.promotions:
        json.dump(make_promotions(a.procs), open(os.path.join(HERE, "perft_promotions.json"), "w"), indent=0)


if __name__ == "__main__":
    main()
