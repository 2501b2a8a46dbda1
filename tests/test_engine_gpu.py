"""Full-engine search on the GB300 against the reference's own
alphabeta_gpu kernel run on the host (refshim): with one worker the GPU
search must visit exactly the reference's tree -- same root score, same PV
(all 64 slots), same node count, TT-move, TT-score and IID-move hits --
with the transposition tables, killer and counter moves carried from one
iterative-deepening depth to the next as the reference host does
(src/search.c:77-198)."""
import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu

# the session fixture's tables: 64 MB of 16-byte TT1 entries, 16 MB of
# 24-byte TT2 entries rounded down to a power of two (src/clrun.c:387-443)
E1, E2 = 1 << 22, 1 << 19
SLOTS = [1, 3, 4, 5]  # nodes, TT-move hits, TT-score hits, IID-move hits


def _need_reference():
    if ol.reference() is None:
        pytest.skip("reference kernels (oracle/_ref) not built")


def _id_compare(z, board, stm, max_depth, ply_init=0, hist=None):
    ref = ol.RefSearch(E1, E2)
    z.tt_clear()
    for d in range(1, max_depth + 1):
        pv_r, c_r = ref.run(board, stm, d, ply_init, hist)
        pv_g, c_g = z.engine_search(board, stm, d, 1, ply_init, hist)
        assert list(pv_g) == list(pv_r), (d, [ol.move2can(m) for m in pv_g[1:8]], [ol.move2can(m) for m in pv_r[1:8]])
        assert list(c_g[0, SLOTS]) == list(c_r[0, SLOTS]), (d, c_g[0, SLOTS], c_r[0, SLOTS])
    return pv_g, c_g


def test_engine_startpos_matches_reference(zeta_device):
    _need_reference()
    b, stm = ol.setboard("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    pv, cnt = _id_compare(zeta_device, b, stm, 6)
    assert np.int32(pv[0]) == 0 and cnt[0, 1] == 16392


def test_engine_depth0_warmup_matches_reference(zeta_device):
    """The reference host's start-up launch cl_run_alphabeta(stm, 0, 1)
    (src/zeta.c:695): a quiescence search of the root, with and without the
    one-node budget, equal to the reference kernel's PV and counters."""
    _need_reference()
    w = zeta_device.WORKLOADS["engine"]
    boards, stm, _ = ol.make_positions(w["seed"], 5, min_plies=w["min_plies"], max_plies=w["max_plies"],
                                       min_pieces=w["min_pieces"], min_depth=0, max_depth=0)
    start, s0 = ol.setboard("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    for b, s in [(start, s0)] + list(zip(boards, stm)):
        for max_nodes in (1, 1 << 40):
            ref = ol.RefSearch(E1, E2)
            zeta_device.tt_clear()
            pv_r, c_r = ref.run(b, int(s), 0, max_nodes=max_nodes)
            pv_g, c_g = zeta_device.engine_search(b, int(s), 0, 1, max_nodes=max_nodes)
            assert list(pv_g) == list(pv_r) and list(c_g[0, SLOTS]) == list(c_r[0, SLOTS]), max_nodes


@pytest.mark.parametrize("i", range(6))
def test_engine_middlegames_match_reference(zeta_device, i):
    _need_reference()
    w = zeta_device.WORKLOADS["engine"]
    boards, stm, _ = ol.make_positions(w["seed"], 6, min_plies=w["min_plies"], max_plies=w["max_plies"],
                                       min_pieces=w["min_pieces"], min_depth=0, max_depth=0)
    _id_compare(zeta_device, boards[i], int(stm[i]), 5)


@pytest.mark.parametrize("fen,depth", [
    ("6k1/5ppp/8/8/8/8/5PPP/3R2K1 w - - 0 1", 6),            # mate in one behind a back rank
    ("8/8/8/8/8/5k2/3p4/5K2 b - - 0 1", 8),                 # promotion: extension, queen moves
    ("8/2p5/3p4/KP5r/1R3p1k/8/4P1P1/8 w - - 0 1", 7),        # en passant, pawn endgame
    ("r3k2r/p1ppqpb1/bn2pnp1/3PN3/1p2P3/2N2Q1p/PPPBBPPP/R3K2R w KQkq - 0 1", 4),  # castles, pins
    ("4k3/8/8/8/8/8/8/4K2R w K - 0 1", 8),                  # rook mate: null move, IID, LMR
    ("8/8/8/8/8/8/k7/2K5 w - - 0 1", 3),                    # bare kings
    ("7k/5Q2/6K1/8/8/8/8/8 b - - 0 1", 3),                  # stalemate
    ("r1bqkbnr/pppp1ppp/2n5/4p3/4P3/5N2/PPPP1PPP/RNBQKB1R w KQkq - 2 3", 7),  # IID at depth 7
])
def test_engine_special_positions_match_reference(zeta_device, fen, depth):
    _need_reference()
    b, stm = ol.setboard(fen)
    _id_compare(zeta_device, b, stm, depth)


def test_engine_repetition_history_matches_reference(zeta_device):
    """A game that returned to the initial position: the search sees the
    earlier occurrences through the hash history (ply_init = 4)."""
    _need_reference()
    b, stm = ol.setboard("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    hist = np.zeros(1024, dtype=np.uint64)
    cur, s = b.copy(), stm
    hist[0] = cur[5]
    for ply, can in enumerate(["g1f3", "g8f6", "f3g1", "f6g8"], start=1):
        mv = ol.can2move(cur, s, can)
        cur = ol.play(cur, s, mv)
        s ^= 1
        hist[ply] = cur[5]
    assert s == stm and int(cur[5]) == int(b[5])
    _id_compare(zeta_device, cur, s, 5, ply_init=4, hist=hist)


def test_engine_batch_matches_single_searches(zeta_device):
    """One launch over 8 positions: each position searches a 1/8 slice of
    the tables and equals the reference with tables of that size."""
    _need_reference()
    z = zeta_device
    w = z.WORKLOADS["engine"]
    boards, stm, _ = ol.make_positions(w["seed"] + 1, 8, min_plies=w["min_plies"], max_plies=w["max_plies"],
                                       min_pieces=w["min_pieces"], min_depth=0, max_depth=0)
    z.tt_clear()
    sc, mv, nodes, pvs = z.engine_batch(boards, stm, 5, 1, with_pv=True)
    for i in range(8):
        ref = ol.RefSearch(E1 // 8, E2 // 8)
        pv_r, c_r = ref.run(boards[i], int(stm[i]), 5)
        assert list(pvs[i]) == list(pv_r), i
        assert sc[i] == np.int32(pv_r[0]) and mv[i] == pv_r[1] and nodes[i] == c_r[0, 1]


def test_engine_workers_share_tables(zeta_device):
    """ABDADA workers: every position finishes, the best move and the PV
    are legal move sequences, and the node counts add up over workers."""
    z = zeta_device
    w = z.WORKLOADS["engine"]
    boards, stm, _ = ol.make_positions(w["seed"] + 2, 4, min_plies=w["min_plies"], max_plies=w["max_plies"],
                                       min_pieces=w["min_pieces"], min_depth=0, max_depth=0)
    z.tt_clear()
    sc, mv, nodes, pvs = z.engine_batch(boards, stm, 7, 16, with_pv=True)
    for i in range(4):
        assert mv[i] != 0 and nodes[i] > 0
        cur, s = boards[i].copy(), int(stm[i])
        for m in pvs[i, 1:]:
            if m == 0:
                break
            assert int(m) in ol.genmoves(cur, s), (i, ol.move2can(int(m)))
            cur = ol.play(cur, s, int(m))
            s ^= 1
        assert pvs[i, 1] == mv[i]


def test_engine_node_budget_stops_the_search(zeta_device):
    z = zeta_device
    b, stm = ol.setboard("r1bqkbnr/pppp1ppp/2n5/4p3/4P3/5N2/PPPP1PPP/RNBQKB1R w KQkq - 2 3")
    z.tt_clear()
    pv, cnt = z.engine_search(b, stm, 12, 1, max_nodes=5000)
    assert cnt[0, 1] == 5001 and not pv.any()  # stopped: no PV, as the reference leaves it


def test_engine_iterative_deepening_matches_reference(zeta_device):
    """zeta_engine_id over 4 positions equals, per position, the reference's
    iterative deepening with tables of a quarter of the size."""
    _need_reference()
    z = zeta_device
    w = z.WORKLOADS["engine"]
    boards, stm, _ = ol.make_positions(w["seed"] + 3, 4, min_plies=w["min_plies"], max_plies=w["max_plies"],
                                       min_pieces=w["min_pieces"], min_depth=0, max_depth=0)
    sc, mv, nodes, dd, *_ = z.engine_id(boards, stm, 6, 1)
    for i in range(4):
        ref = ol.RefSearch(E1 // 4, E2 // 4)
        total = 0
        for d in range(1, 7):
            pv_r, c_r = ref.run(boards[i], int(stm[i]), d)
            total += int(c_r[0, 1])
        assert dd[i] == 6 and sc[i] == np.int32(pv_r[0]) and mv[i] == pv_r[1] and nodes[i] == total, i


def test_engine_learned_ordering_runs(zeta_device):
    """The network orders quiet moves: the search still returns legal best
    moves, and the network's time is accounted."""
    z = zeta_device
    z.mlp_init(3)
    w = z.WORKLOADS["engine"]
    boards, stm, _ = ol.make_positions(w["seed"] + 4, 16, min_plies=w["min_plies"], max_plies=w["max_plies"],
                                       min_pieces=w["min_pieces"], min_depth=0, max_depth=0)
    for ordering in (1, 2):
        sc, mv, nodes, dd, ms, ms_s, ms_n = z.engine_id(boards, stm, 6, 4, ordering)
        assert (dd >= 1).all() and ms_n > 0
        for i in range(16):
            assert int(mv[i]) in ol.genmoves(boards[i], int(stm[i]))


@pytest.mark.parametrize("form", [1, 2])
def test_engine_launch_forms_match_reference(zeta_device, form):
    """Dense and sparse launches of an 8-position batch with one worker
    each: every position equals the reference's search exactly."""
    _need_reference()
    z = zeta_device
    w = z.WORKLOADS["engine"]
    boards, stm, _ = ol.make_positions(w["seed"] + 3, 8, min_plies=w["min_plies"], max_plies=w["max_plies"],
                                       min_pieces=w["min_pieces"], min_depth=0, max_depth=0)
    z.search_set_launch_form(form)
    try:
        z.tt_clear()
        sc, mv, nodes, pvs = z.engine_batch(boards, stm, 5, 1, with_pv=True)
    finally:
        z.search_set_launch_form(0)
    for i in range(8):
        ref = ol.RefSearch(E1 // 8, E2 // 8)
        pv_r, c_r = ref.run(boards[i], int(stm[i]), 5)
        assert list(pvs[i]) == list(pv_r), (form, i)
        assert sc[i] == np.int32(pv_r[0]) and mv[i] == pv_r[1] and nodes[i] == c_r[0, 1]


def test_engine_deeper_helpers(zeta_device):
    """Lazy SMP (no TT2) with every second helper one ply deeper
    (zeta_engine_set_helper_depth): worker 0 -- and so a one-worker search
    -- still visits exactly the reference's tree, and a 16-worker
    iterative deepening ends every depth with a legal PV from a worker at
    that depth."""
    _need_reference()
    z = zeta_device
    z.release()
    z.init(0, 64, 0)
    try:
        z.engine_set_helper_depth(2)
        b, stm = ol.setboard("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
        ref = ol.RefSearch(E1, 0)
        z.tt_clear()
        for d in range(1, 6):
            pv_r, c_r = ref.run(b, stm, d)
            pv_g, c_g = z.engine_search(b, stm, d, 1)
            assert list(pv_g) == list(pv_r) and list(c_g[0, SLOTS]) == list(c_r[0, SLOTS]), d
        w = z.WORKLOADS["engine"]
        boards, stms, _ = ol.make_positions(w["seed"] + 3, 2, min_plies=w["min_plies"], max_plies=w["max_plies"],
                                            min_pieces=w["min_pieces"], min_depth=0, max_depth=0)
        for i in range(2):
            z.tt_clear()
            for d in range(1, 8):
                pv, cnt = z.engine_search(boards[i], int(stms[i]), d, 16)
                assert pv[1] != 0 and cnt[:, 1].sum() > 0, (i, d)
                cur, s = boards[i].copy(), int(stms[i])
                for m in pv[1:1 + d]:
                    if m == 0:
                        break
                    assert int(m) in ol.genmoves(cur, s), (i, d, ol.move2can(int(m)))
                    cur = ol.play(cur, s, int(m))
                    s ^= 1
        with pytest.raises(z.ZetaError):
            z.engine_set_helper_depth(1)
    finally:
        z.engine_set_helper_depth(0)
        z.release()
        z.init(0, 64, 16)
