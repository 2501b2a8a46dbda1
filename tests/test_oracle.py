"""The oracle against the reference's own pins (CPU only)."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle_lib as ol

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return json.load(open(os.path.join(GOLD, name)))


def board_of(case):
    return np.array([int(x, 16) for x in case["board"]], dtype=np.uint64)


@pytest.mark.parametrize("case", load("perft_kat.json"), ids=lambda c: f"{c['fen'][:12]}-d{c['depth']}")
def test_oracle_selftest_kats(case):
    """The 14 known-answer tests of src/test.c:43-73."""
    b, stm = ol.setboard(case["fen"])
    assert ol.perft(b, stm, case["depth"]) == case["leaves"]


def test_oracle_matches_reference_kernel_counts():
    """Leaf counts of the unmodified reference perft kernel (tests/golden/perft_ref.json)."""
    cases = [c for c in load("perft_ref.json") if c["leaves"] < 3_000_000]
    bad = [c["name"] for c in cases if ol.perft(board_of(c), c["stm"], c["depth"]) != c["leaves"]]
    assert not bad, bad[:10]
    kinds = {c["name"].rstrip("0123456789-d").rstrip("0123456789") for c in cases}
    assert {"random", "promo", "ep", "castle"} <= kinds


def test_oracle_tables_equal_reference_literals():
    ref = load("tables.json")
    for key, fn, n in (("AttackTablesPawnPushes", "zo_pawn_push_tables", 128),
                       ("AttackTables", "zo_attack_tables", 448),
                       ("bbInBetween", "zo_inbetween_table", 4096),
                       ("bbLine", "zo_line_table", 4096)):
        t = ol.table(fn, n).astype("<u8")
        assert hashlib.sha256(t.tobytes()).hexdigest() == ref[key], key


def test_setboard_fen_ep_square_is_ignored_like_the_reference():
    """setboard clears the flag of the FEN target square (rank 3/6), outside
    the engine's rank-4/5 en-passant mask (src/io.c:495-505)."""
    b1, s1 = ol.setboard("rnbqkbnr/ppp1pppp/8/3pP3/8/8/PPPP1PPP/RNBQKBNR w KQkq d6 0 3")
    b2, s2 = ol.setboard("rnbqkbnr/ppp1pppp/8/3pP3/8/8/PPPP1PPP/RNBQKBNR w KQkq - 0 3")
    assert ol.perft(b1, s1, 1) == ol.perft(b2, s2, 1)
    assert not any((m >> 12) & 63 != (m >> 6) & 63 and (m >> 18) >> 1 & 7 == 1 for m in ol.genmoves(b1, s1))


def test_hash_of_initial_position_and_incremental_agree():
    b, s = ol.setboard("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    assert int(b[5]) == ol.computehash(b, s)
    # the search kernel's incremental hash equals a full rehash after a normal move
    for m in ol.genmoves(b, s):
        c = ol.play(b, s, m)
        assert int(c[5]) == ol.computehash(c, 1 - s)


def test_negamax_equals_alphabeta():
    pos = [ol.make_position(7, i, 20, 40, 20, 2, 3) for i in range(6)]
    for b, s, d in pos:
        v1, m1, n1 = ol.negamax(b, s, d)
        v2, m2, n2 = ol.alphabeta(b, s, d)
        assert v1 == v2
        assert n2 <= n1


def test_position_generator_is_deterministic_and_legal():
    a = ol.make_positions(123, 16, min_plies=10, max_plies=60, min_depth=3, max_depth=5)
    b = ol.make_positions(123, 16, min_plies=10, max_plies=60, min_depth=3, max_depth=5)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    boards, stm, depth = a
    assert set(depth.tolist()) <= {3, 4, 5}
    for i in range(16):
        assert ol.movecount(boards[i], stm[i])[0] > 0
        assert int(boards[i][5]) == ol.computehash(boards[i], stm[i])
