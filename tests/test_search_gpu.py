"""Batched pure fixed-depth search on the GB300 against the oracle's plain
negamax / alpha-beta (integer scores: exact equality)."""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu


def _positions(seed, n, lo=10, hi=60, pieces=0):
    return ol.make_positions(seed, n, min_plies=lo, max_plies=hi, min_pieces=pieces, min_depth=0, max_depth=0)


@pytest.mark.parametrize("depth", [1, 2, 3, 4])
def test_root_scores_equal_negamax(zeta_device, depth):
    z = zeta_device
    boards, stm, _ = _positions(0x5EA7C0 + depth, 96, 1, 120)
    for workers in (1, 4):
        z.tt_clear()
        scores, moves, nodes = z.search_batch(boards, stm, depth, workers)
        for i in range(len(stm)):
            v, _, _ = ol.alphabeta(boards[i], stm[i], depth)
            assert scores[i] == v, (i, depth, workers, scores[i], v)
        assert (nodes > 0).all()


def test_best_move_reaches_the_score(zeta_device):
    z = zeta_device
    depth = 3
    boards, stm, _ = _positions(0xB357, 48, 10, 60)
    z.tt_clear()
    scores, moves, _ = z.search_batch(boards, stm, depth, 4)
    for i in range(len(stm)):
        legal = ol.genmoves(boards[i], stm[i])
        assert moves[i] in legal
        child = ol.play(boards[i], stm[i], int(moves[i]))
        v, _, _ = ol.alphabeta(child, 1 - stm[i], depth - 1)
        # the child is one ply deeper: shift its mate distance by one ply
        if abs(v) > 30000:
            v = v - 1 if v > 0 else v + 1
        assert -v == scores[i], i


def test_mate_and_stalemate_scores(zeta_device):
    z = zeta_device
    mate_in_1, s1 = ol.setboard("6k1/5ppp/8/8/8/8/5PPP/3R2K1 w - - 0 1")   # Rd8#
    mated, s2 = ol.setboard("rnb1kbnr/pppp1ppp/8/4p3/6Pq/5P2/PPPPP2P/RNBQKBNR w KQkq - 1 3")
    stale, s3 = ol.setboard("7k/5Q2/6K1/8/8/8/8/8 b - - 0 1")
    boards = np.stack([mate_in_1, mated, stale])
    stm = np.array([s1, s2, s3], np.uint8)
    for depth in (1, 2, 3):
        z.tt_clear()
        scores, _, _ = z.search_batch(boards, stm, depth, 2)
        want = [ol.alphabeta(boards[i], stm[i], depth)[0] for i in range(3)]
        assert list(scores) == want, depth
    assert want[0] == 32000 - 1 and want[1] == -32000 and want[2] == 0


def test_deeper_search_matches_oracle_and_worker_counts_agree(zeta_device):
    z = zeta_device
    boards, stm, _ = _positions(0xD5, 6, 20, 40, 20)
    want = [ol.alphabeta(boards[i], stm[i], 5)[0] for i in range(len(stm))]
    for workers in (1, 3, 8, 16):
        z.tt_clear()
        scores, _, _ = z.search_batch(boards, stm, 5, workers)
        assert list(scores) == want, workers
    # a warm table (entries of the previous calls) does not change values
    scores, _, _ = z.search_batch(boards, stm, 5, 8)
    assert list(scores) == want


def test_benchmark_workload_depth7_is_worker_independent(zeta_device):
    """Full benchmark depth on a sample: values agree across worker counts
    and with a cold or warm table (size-independent check)."""
    z = zeta_device
    w = z.WORKLOADS["search_batch"]
    boards, stm, _ = z.make_positions(w["seed"], 64, w["min_plies"], w["max_plies"], w["min_pieces"], 0, 0)
    z.tt_clear()
    a, _, _ = z.search_batch(boards, stm, 7, 1)
    z.tt_clear()
    b, _, _ = z.search_batch(boards, stm, 7, 8)
    c, _, _ = z.search_batch(boards, stm, 7, 8)
    assert np.array_equal(a, b) and np.array_equal(b, c)


@pytest.mark.parametrize("form", [1, 2, 3])
def test_launch_forms_give_the_same_scores(zeta_device, form):
    """Dense (32 workers per warp), sparse (one per warp) and warp-cooperative
    (one worker per warp whose lanes score the last ply together) launches
    of the same batch: root scores equal the oracle's negamax in all."""
    z = zeta_device
    boards, stm, _ = _positions(0xF0A11 + form, 40, 10, 80)
    want = [ol.alphabeta(boards[i], stm[i], 4)[0] for i in range(len(stm))]
    z.search_set_launch_form(form)
    try:
        for workers in (1, 5):
            z.tt_clear()
            scores, moves, nodes = z.search_batch(boards, stm, 4, workers)
            assert list(scores) == want, (form, workers)
            assert (nodes > 0).all()
            # table operations counted on the device: each node entered
            # probes at most once and each finished node stores once
            probes, stores = z.search_last_table_ops()
            assert 0 < stores <= probes + len(stm) * workers and probes + stores <= 2 * int(nodes.sum()), \
                (form, workers, probes, stores, int(nodes.sum()))
    finally:
        z.search_set_launch_form(0)


def test_warp_form_depths_mates_best_moves_and_helpers(zeta_device):
    """The warp-cooperative form at depths 1-5 (depth 1: the root itself
    is scored by the lanes), with mated, stalemated and mate-in-one roots,
    several workers and helpers: root scores equal negamax, and the best
    move's child has the root's value."""
    z = zeta_device
    boards, stm, _ = _positions(0x3A4B, 24, 10, 90)
    extra = [ol.setboard(f) for f in ("6k1/5ppp/8/8/8/8/5PPP/3R2K1 w - - 0 1",
                                      "rnb1kbnr/pppp1ppp/8/4p3/6Pq/5P2/PPPPP2P/RNBQKBNR w KQkq - 1 3",
                                      "7k/5Q2/6K1/8/8/8/8/8 b - - 0 1")]
    boards = np.concatenate([boards, np.stack([b for b, _ in extra])])
    stm = np.concatenate([stm, np.array([s for _, s in extra], np.uint8)])
    z.search_set_launch_form(3)
    try:
        for depth in (1, 2, 3, 4, 5):
            want = [ol.alphabeta(boards[i], stm[i], depth)[0] for i in range(len(stm))]
            for workers, helpers in ((1, 0), (3, 0), (1, 4)):
                z.search_set_helpers(helpers)
                z.tt_clear()
                scores, moves, nodes = z.search_batch(boards, stm, depth, workers)
                assert list(scores) == want, (depth, workers, helpers)
                assert (nodes > 0).all()
            if depth <= 3:
                for i in range(len(stm)):
                    legal = ol.genmoves(boards[i], stm[i])
                    if not legal:
                        assert moves[i] == 0
                        continue
                    assert moves[i] in legal
                    child = ol.play(boards[i], stm[i], int(moves[i]))
                    v = ol.alphabeta(child, 1 - stm[i], depth - 1)[0] if depth > 1 else None
                    if v is None:
                        continue
                    if abs(v) > 30000:
                        v = v - 1 if v > 0 else v + 1
                    assert -v == scores[i], (depth, i)
    finally:
        z.search_set_launch_form(0)
        z.search_set_helpers(0)


def test_device_evaluation_matches_oracle(zeta_device):
    """The device evaluation (white's view) equals the oracle's restatement
    of the reference evaluation on every board: playouts of all lengths,
    the benchmark workload, and the special positions."""
    z = zeta_device
    boards, stm, _ = _positions(0xE7A1, 20000, 1, 200)
    w = z.WORKLOADS["search_batch"]
    wb, _, _ = z.make_positions(w["seed"], 2000, w["min_plies"], w["max_plies"], w["min_pieces"], 0, 0)
    special = [ol.setboard(f)[0] for f in (
        "rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1",
        "r3k2r/Pppp1ppp/1b3nbN/nP6/BBP1P3/q4N2/Pp1P2PP/R2Q1RK1 w kq - 0 1",
        "8/2p5/3p4/KP5r/1R3p1k/8/4P1P1/8 w - - 0 1",
        "4k3/8/8/8/8/8/8/4K2R w K - 0 1",
        "2b1kb2/8/8/8/8/8/8/2B1KB2 w - - 0 1")]                  # both bishop pairs
    allb = np.concatenate([boards, wb, np.stack(special)])
    got = z.eval_batch(allb)
    want = np.array([ol.eval_white(b) for b in allb])
    bad = np.nonzero(got != want)[0]
    assert len(bad) == 0, (len(bad), bad[:5].tolist(), got[bad[:5]].tolist(), want[bad[:5]].tolist())
