"""Promotion to a rook, bishop or knight, a rule the reference does not
have (zetaperft.cl:1380-1384 promotes to a queen only), so nothing of the
reference can pin it.  The pin is a second generator that shares no code
or method with the oracle: tests/mailbox_gen.py walks a 64-square mailbox
and tests each pseudo-legal move for king safety.  With queen-only
promotions it must reproduce the oracle, which the reference's own counts
pin (tests/golden/perft_ref.json); with all four promotions it must
reproduce the oracle's all-promotions mode (zo_genmoves_ex, zo_perft_ex)."""
import json
import os

import numpy as np
import pytest

import mailbox_gen as mb
import oracle_lib as ol

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "perft_promotions.json")


def _fixture():
    with open(FIXTURE) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def random_positions():
    return ol.make_positions(0xB0B, 400, min_plies=1, max_plies=160)


def test_mailbox_equals_oracle_move_for_move(random_positions):
    boards, stm, _ = random_positions
    promoting = 0
    for i in range(len(stm)):
        q = sorted(ol.genmoves(boards[i], stm[i]))
        assert sorted(mb.board_moves(boards[i], stm[i])) == q, i
        a = sorted(ol.genmoves(boards[i], stm[i], all_promotions=True))
        assert sorted(mb.board_moves(boards[i], stm[i], True)) == a, i
        promoting += len(a) != len(q)
    assert promoting >= 10, promoting  # the sample does exercise the rule


def test_all_promotion_moves_follow_each_queen_promotion(random_positions):
    boards, stm, _ = random_positions
    for i in range(len(stm)):
        q = ol.genmoves(boards[i], stm[i])
        a = ol.genmoves(boards[i], stm[i], all_promotions=True)
        promos = [m for m in q if ((m >> 18) & 15) >> 1 == 1 and ((m >> 22) & 15) >> 1 == 6]
        assert len(a) == len(q) + 3 * len(promos)
        for m in promos:
            rest = m & ~(15 << 22)
            side = (m >> 18) & 1
            for kind in (5, 4, 2):  # rook, bishop, knight
                assert rest | ((kind << 1 | side) << 22) in a
        # captures only: the same rule on the capture list
        qc = ol.genmoves(boards[i], stm[i], qs=True)
        ac = ol.genmoves(boards[i], stm[i], qs=True, all_promotions=True)
        assert len(ac) == len(qc) + 3 * sum(1 for m in qc if ((m >> 22) & 15) >> 1 == 6 and ((m >> 18) & 15) >> 1 == 1)


def test_mailbox_perft_equals_oracle_on_promoting_positions(random_positions):
    boards, stm, _ = random_positions
    picked = [i for i in range(len(stm))
              if len(ol.genmoves(boards[i], stm[i], all_promotions=True)) != len(ol.genmoves(boards[i], stm[i]))][:6]
    assert picked
    for i in picked:
        for ap in (False, True):
            assert mb.board_perft(boards[i], stm[i], 3, ap) == ol.perft(boards[i], stm[i], 3, ap), (i, ap)


def test_hand_made_positions_match_fixture():
    fx = _fixture()
    assert len(fx["special"]) == 5
    for row in fx["special"]:
        b, s = ol.setboard(row["fen"])
        for d in range(1, 4):
            assert ol.perft(b, s, d) == row["queen_only"][d - 1], (row["fen"], d)
            assert ol.perft(b, s, d, all_promotions=True) == row["all_promotions"][d - 1], (row["fen"], d)
            assert mb.board_perft(b, s, d, True) == row["all_promotions"][d - 1], (row["fen"], d)
        assert row["all_promotions"][-1] > row["queen_only"][-1]


def test_workload_fixture_is_consistent_with_the_queen_only_fixture():
    fx = _fixture()
    with open(os.path.join(HERE, "golden", "perft_workload.json")) as f:
        queen = json.load(f)
    assert fx["positions_sha256"] == queen["positions_sha256"]
    assert len(fx["leaves"]) == len(queen["leaves"]) == 4096
    differ = [i for i in range(4096) if fx["leaves"][i] != queen["leaves"][i]]
    assert differ == fx["differ_from_queen_only"] and differ
    # more promotion choices never remove a leaf
    assert all(fx["leaves"][i] > queen["leaves"][i] for i in differ)
    assert fx["total_leaves"] == sum(fx["leaves"])


def test_oracle_reproduces_workload_fixture_sample():
    fx = _fixture()
    w = fx["workload"]
    boards, stm, depth = ol.make_positions(int(w["seed"], 16), 4096, min_plies=w["min_plies"],
                                           max_plies=w["max_plies"], min_pieces=w["min_pieces"],
                                           min_depth=w["min_depth"], max_depth=w["max_depth"])
    sample = [i for i in fx["differ_from_queen_only"] if depth[i] == 3][:8]
    assert sample
    for i in sample:
        assert ol.perft(boards[i], stm[i], 3, all_promotions=True) == fx["leaves"][i], i


def test_two_pawns_promoting_on_the_same_square():
    """Two pawns that can take the same piece on the last rank make two
    capture promotions of each kind (eight moves, not four)."""
    for fen in ("2r4k/1P1P4/8/8/8/8/8/4K3 w - - 0 1", "4k3/8/8/8/8/8/1p1p4/2R3K1 b - - 0 1"):
        b, s = ol.setboard(fen)
        caps = [m for m in ol.genmoves(b, s, qs=True, all_promotions=True) if ((m >> 18) & 15) >> 1 == 1]
        assert len(caps) == 8 and len({m & 63 for m in caps}) == 2, fen
        for d in range(1, 4):
            assert mb.board_perft(b, s, d, True) == ol.perft(b, s, d, all_promotions=True), (fen, d)
