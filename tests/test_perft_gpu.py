"""Perft on the GB300 through the C ABI, checked against the reference's
known answers, the reference kernels' own counts (golden fixtures) and the
oracle.  Integer work: every comparison is bit-exact."""
import json
import os

import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return json.load(open(os.path.join(GOLD, name)))


def board_of(case):
    return np.array([int(x, 16) for x in case["board"]], dtype=np.uint64)


def test_selftest_kats(zeta_device):
    """src/test.c:43-73, one call per KAT as selftest() does."""
    z = zeta_device
    for case in load("perft_kat.json"):
        b, stm = ol.setboard(case["fen"])
        assert z.perft(b, stm, case["depth"]) == case["leaves"], case


def test_reference_kernel_counts_batched(zeta_device):
    """Every fixture made by the unmodified reference kernel, in one batch."""
    z = zeta_device
    cases = load("perft_ref.json")
    boards = np.stack([board_of(c) for c in cases])
    stm = np.array([c["stm"] for c in cases], dtype=np.uint8)
    depth = np.array([c["depth"] for c in cases], dtype=np.uint8)
    got = z.perft_batch(boards, stm, depth)
    want = np.array([c["leaves"] for c in cases], dtype=np.uint64)
    bad = [(cases[i]["name"], int(got[i]), int(want[i])) for i in np.nonzero(got != want)[0]]
    assert not bad, bad[:10]


def test_startpos_depth6(zeta_device):
    """Depth 6 of the initial position: the headline single-position case."""
    z = zeta_device
    b, s = ol.setboard("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    assert z.perft(b, s, 6) == 119060324


def test_random_positions_vs_oracle(zeta_device):
    z = zeta_device
    boards, stm, depth = ol.make_positions(0xBEEF, 200, min_plies=1, max_plies=150, min_depth=1, max_depth=3)
    got = z.perft_batch(boards, stm, depth)
    want = np.array([ol.perft(boards[i], stm[i], depth[i]) for i in range(len(depth))], dtype=np.uint64)
    assert np.array_equal(got, want)


def test_edge_depths_and_terminal_positions(zeta_device):
    z = zeta_device
    b, s = ol.setboard("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    assert z.perft(b, s, 0) == 1
    assert z.perft(b, s, 1) == 20
    mate, ms = ol.setboard("rnb1kbnr/pppp1ppp/8/4p3/6Pq/5P2/PPPPP2P/RNBQKBNR w KQkq - 1 3")
    stale, ss = ol.setboard("7k/5Q2/6K1/8/8/8/8/8 b - - 0 1")
    for d in (1, 2, 3):
        assert z.perft(mate, ms, d) == 0
        assert z.perft(stale, ss, d) == 0
    assert z.perft(mate, ms, 0) == 1


def test_bad_arguments_are_rejected(zeta_device):
    z = zeta_device
    b = np.array(z.STARTPOS)
    with pytest.raises(z.ZetaError):
        z.perft(b, 0, 99)
    with pytest.raises(ValueError):
        z.perft_batch(np.stack([b, b]), np.zeros(1, np.uint8), np.ones(2, np.uint8))


def test_launch_shapes_do_not_change_counts(zeta_device):
    """Block size, split policy and graph replay are scheduling only."""
    z = zeta_device
    boards, stm, depth = ol.make_positions(0xC0FFEE, 64, min_plies=10, max_plies=60, min_depth=2, max_depth=4)
    base = z.perft_batch(boards, stm, depth)
    from zeta_gb300.autotune import VARIANTS
    saved = z.perft_config()
    try:
        for tpb, bps in VARIANTS:
            for td in (1, 2, 3, 4):
                z.perft_configure(threads_per_block=tpb, blocks_per_sm=bps, task_depth=td)
                assert np.array_equal(z.perft_batch(boards, stm, depth), base), (tpb, bps, td)
        for mt in (0, 1000, 10**6):
            for graph in (True, False):
                z.perft_configure(threads_per_block=128, task_depth=3, min_tasks=mt, use_graph=graph)
                assert np.array_equal(z.perft_batch(boards, stm, depth), base), (mt, graph)
        with pytest.raises(z.ZetaError):
            z.perft_configure(threads_per_block=128, blocks_per_sm=5, task_depth=3)
            z.perft_batch(boards, stm, depth)
    finally:
        z.perft_configure(**saved)


def test_graph_replay_is_repeatable(zeta_device):
    z = zeta_device
    boards, stm, depth = ol.make_positions(0xFACE, 300, min_plies=10, max_plies=60, min_depth=3, max_depth=4)
    first = z.perft_batch(boards, stm, depth)
    for _ in range(3):
        assert np.array_equal(z.perft_batch(boards, stm, depth), first)
    st = z.perft_stats()
    assert st["tasks"] > 0 and st["counted_nodes"] > 0


def test_batch_workload_sample_vs_reference_sum_of_children(zeta_device):
    """Size-independent check at the benchmark's depths: a position's count
    equals the sum of its children's counts one ply shallower."""
    z = zeta_device
    w = dict(z.WORKLOADS["perft_batch"])
    boards, stm, depth = z.make_positions(w["seed"], 24, w["min_plies"], w["max_plies"], w["min_pieces"],
                                          w["min_depth"], w["max_depth"])
    whole = z.perft_batch(boards, stm, depth)
    for i in range(len(depth)):
        kids = [ol.play(boards[i], stm[i], m, perft_flags=True) for m in ol.genmoves(boards[i], stm[i])]
        if not kids:
            assert whole[i] == 0
            continue
        sub = z.perft_batch(np.stack(kids), np.full(len(kids), 1 - stm[i], np.uint8),
                            np.full(len(kids), depth[i] - 1, np.uint8))
        assert int(sub.sum()) == int(whole[i])


@pytest.mark.parametrize("generator", [0, 1, 2])
def test_genmoves_matches_oracle(zeta_device, generator):
    """Each device generator (perft, search kernels, warp-cooperative
    search) gives the oracle's legal set, move for move in the reference
    packing; the warp generator gives the search kernels' list in the same
    order."""
    z = zeta_device
    boards, stm, _ = ol.make_positions(0xD00D, 400, min_plies=1, max_plies=200)
    special = [ol.setboard(f) for f in (
        "r3k2r/p1ppqpb1/bn2pnp1/3PN3/1p2P3/2N2Q1p/PPPBBPPP/R3K2R w KQkq - 0 1",   # castles, pins
        "8/2p5/3p4/KP5r/1R3p1k/8/4P1P1/8 w - - 0 1",                             # en passant, pins
        "r3k2r/Pppp1ppp/1b3nbN/nP6/BBP1P3/q4N2/Pp1P2PP/R2Q1RK1 w kq - 0 1",      # promotions, checks
        "rnbq1k1r/pp1Pbppp/2p5/8/2B5/8/PPP1NnPP/RNBQK2R w KQ - 1 8",             # promotion captures
        "4k3/8/8/8/8/8/8/4K2R w K - 0 1",
        "8/8/8/8/8/5k2/3p4/5K2 b - - 0 1",
        "R6r/8/8/2K5/5k2/8/8/r6R w - - 0 1",                                     # rook pins
        "3k4/3p4/8/K1P4r/8/8/8/8 b - - 0 1",                                     # double push, ep pin
        "8/8/1k6/2b5/2pP4/8/5K2/8 b - d3 0 1",                                   # ep capture
        "7k/5Q2/6K1/8/8/8/8/8 b - - 0 1",                                        # stalemate
        "rnb1kbnr/pppp1ppp/8/4p3/6Pq/5P2/PPPPP2P/RNBQKBNR w KQkq - 1 3")]        # mate
    boards = np.concatenate([boards, np.stack([b for b, _ in special])])
    stm = np.concatenate([stm, np.array([s for _, s in special], np.uint8)])
    for qs in (False, True):
        lists = z.genmoves_batch(boards, stm, qs=qs, generator=generator)
        for i in range(len(stm)):
            assert sorted(lists[i].tolist()) == sorted(ol.genmoves(boards[i], stm[i], qs)), (generator, qs, i)
        if generator == 2:
            serial = z.genmoves_batch(boards, stm, qs=qs, generator=1)
            for i in range(len(stm)):
                assert lists[i].tolist() == serial[i].tolist(), (qs, i)


def test_device_positions_match_oracle_generator(zeta_device):
    z = zeta_device
    for name in ("perft_batch", "search_batch"):
        w = dict(z.WORKLOADS[name])
        n = 64
        gb, gs, gd = z.make_positions(w["seed"], n, w["min_plies"], w["max_plies"], w["min_pieces"],
                                      w["min_depth"], w["max_depth"])
        ob, os_, od = ol.make_positions(w["seed"], n, min_plies=w["min_plies"], max_plies=w["max_plies"],
                                        min_pieces=w["min_pieces"], min_depth=w["min_depth"],
                                        max_depth=w["max_depth"])
        assert np.array_equal(gb, ob) and np.array_equal(gs, os_) and np.array_equal(gd, od), name
