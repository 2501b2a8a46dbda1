"""Make the golden fixtures of tests/golden/ from the reference itself.

Run in a container that holds the reference tree (default /root/reference)
after ``make -C oracle ref`` has built the reference kernels for the host:

    python tests/golden/make_golden.py [--reference /root/reference]

Fixtures written (all small JSON):
  perft_kat.json   the 14 perft known-answer tests of src/test.c:43-73,
                   read from that file as text
  tables.json      SHA-256 of the reference's literal move-generation
                   tables (zetaperft.cl AttackTables/AttackTablesPawnPushes,
                   bitboard.c bbInBetween/bbLine), so a test can check the
                   oracle's derived tables without copying them
  perft_ref.json   leaf counts computed by the reference perft kernel
                   (oracle/_ref, unmodified zetaperft.cl on host cores) for
                   seeded random positions, promotion and en-passant cases
                   and the initial position to depth 5
  search_ref.json  root score, best move and node counters of the
                   reference search kernel (unmodified zeta.cl, one worker)
                   on seeded positions, when --search is given
Nothing here is read at test time except the JSON files.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import re
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import oracle_lib as ol  # noqa: E402


def hexb(board) -> list[str]:
    return ["0x%016x" % int(x) for x in board]


def kats(ref: str) -> list[dict]:
    text = open(os.path.join(ref, "src", "test.c")).read()
    fens = re.findall(r'"([^"]+/[^"]+)"', text[text.index("fenpositions"):text.index("u32 depths")])
    dsec = text[text.index("u32 depths"):text.index("u64 nodecounts")]
    depths = [int(x) for x in re.findall(r"\b(\d+)\b", dsec.split("=", 1)[1])]
    nsec = text[text.index("u64 nodecounts"):]
    nsec = nsec[nsec.index("{") + 1:nsec.index("}")]
    counts = [int(x) for x in re.findall(r"\b(\d+)\b", nsec)]
    assert len(fens) == len(depths) == len(counts) == 14, (len(fens), len(depths), len(counts))
    return [{"fen": f.strip(), "depth": d, "leaves": c, "source": "src/test.c:43-73"}
            for f, d, c in zip(fens, depths, counts)]


def table_hashes(ref: str) -> dict:
    out = {}
    cl = open(os.path.join(ref, "src", "zetaperft.cl")).read()
    bb = open(os.path.join(ref, "src", "bitboard.c")).read()

    def grab(src: str, name: str) -> list[int]:
        i = src.index(name)
        body = src[src.index("{", i) + 1:src.index("};", i)]
        return [int(x, 16) for x in re.findall(r"0x[0-9a-fA-F]+", body)]

    for key, src, name, n in (("AttackTablesPawnPushes", cl, "AttackTablesPawnPushes[2*64]", 128),
                              ("AttackTables", cl, "AttackTables[7*64]", 448),
                              ("bbInBetween", bb, "bbInBetween[64*64]", 4096),
                              ("bbLine", bb, "bbLine[64*64]", 4096)):
        vals = grab(src, name)
        assert len(vals) == n, (key, len(vals))
        out[key] = hashlib.sha256(np.array(vals, dtype="<u8").tobytes()).hexdigest()
    return out


def random_positions(seed: int, n: int, lo: int, hi: int):
    st = [seed]

    def nxt() -> int:
        st[0] = (st[0] + 0x9E3779B97F4A7C15) & (2**64 - 1)
        z = st[0]
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & (2**64 - 1)
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & (2**64 - 1)
        return z ^ (z >> 31)

    out = []
    while len(out) < n:
        plies = lo + nxt() % (hi - lo + 1)
        r = ol.playout(nxt(), plies)
        if r is not None and ol.movecount(*r)[0] > 0:
            out.append(r)
    return out


def has_kind(board, stm, kind: str) -> bool:
    for m in ol.genmoves(board, stm):
        pf, pt = (m >> 18) & 15, (m >> 22) & 15
        to, cpt = (m >> 6) & 63, (m >> 12) & 63
        if kind == "promo" and (pf >> 1) == 1 and (pt >> 1) == 6:
            return True
        if kind == "ep" and (pf >> 1) == 1 and cpt != to:
            return True
        if kind == "castle" and (pf >> 1) == 3 and abs((m & 63) - to) == 2:
            return True
    return False


def perft_cases() -> list[dict]:
    cases = []
    start, s0 = ol.setboard("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    for d in range(1, 6):
        t = time.time()
        cases.append({"name": f"startpos-d{d}", "board": hexb(start), "stm": s0, "depth": d,
                      "leaves": ol.ref_perft(start, s0, d, threads=os.cpu_count() or 8)})
        print(cases[-1]["name"], cases[-1]["leaves"], "%.1fs" % (time.time() - t), flush=True)
    # seeded random playouts, every phase of the game
    pos = random_positions(0xA11CE, 96, 1, 160)
    boards = np.array([p[0] for p in pos])
    stms = np.array([p[1] for p in pos])
    for d in (1, 2, 3):
        leaves = ol.ref_perft_batch(boards, stms, np.full(len(pos), d), os.cpu_count() or 8)
        for i, (b, s) in enumerate(pos):
            cases.append({"name": f"random{i}-d{d}", "board": hexb(b), "stm": int(s), "depth": d,
                          "leaves": int(leaves[i])})
    # positions where a promotion, an en-passant capture or a castle is legal now
    for kind, want in (("promo", 24), ("ep", 16), ("castle", 16)):
        found = []
        seed = {"promo": 0xB0B, "ep": 0xE9, "castle": 0xCA57}[kind]
        lo, hi = {"promo": (60, 220), "ep": (4, 40), "castle": (6, 30)}[kind]
        for b, s in random_positions(seed, 6000, lo, hi):
            if has_kind(b, s, kind):
                found.append((b, s))
                if len(found) == want:
                    break
        boards = np.array([p[0] for p in found])
        stms = np.array([p[1] for p in found])
        for d in (1, 2, 3):
            leaves = ol.ref_perft_batch(boards, stms, np.full(len(found), d), os.cpu_count() or 8)
            for i, (b, s) in enumerate(found):
                cases.append({"name": f"{kind}{i}-d{d}", "board": hexb(b), "stm": int(s), "depth": d,
                              "leaves": int(leaves[i])})
        print(kind, len(found), flush=True)
    return cases


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--search", action="store_true", help="also make search_ref.json")
    ap.add_argument("--skip-perft", action="store_true")
    a = ap.parse_args()
    if ol.reference() is None:
        sys.exit("build the reference kernels first: make -C oracle ref")
    json.dump(kats(a.reference), open(os.path.join(HERE, "perft_kat.json"), "w"), indent=1)
    json.dump(table_hashes(a.reference), open(os.path.join(HERE, "tables.json"), "w"), indent=1)
    if not a.skip_perft:
        json.dump(perft_cases(), open(os.path.join(HERE, "perft_ref.json"), "w"), indent=0)
    if a.search:
        import make_search_golden
        make_search_golden.main()


if __name__ == "__main__":
    main()
