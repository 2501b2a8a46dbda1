"""Promotion to any of the four pieces on the GB300 (a rule the reference
does not have; its perft promotes to a queen only, zetaperft.cl:1380-1384).

* the perft generator with genmoves flag bit 3 gives the oracle's
  all-promotions move set (zo_genmoves_ex), all moves and captures only;
* zeta_perft_set_promotions(1): the whole 4096-position perft bench batch
  at its drawn depths 3-5 equals the oracle's all-promotions counts
  (tests/golden/perft_promotions.json, cross-checked there by an
  independent mailbox generator), and switching back gives the
  reference's queen-only counts again;
* the allocation-free entry and the host binary (`zeta -u`, the
  `promotions` command) follow the same rule.
The oracle and the mailbox generator (tests/mailbox_gen.py) pin the rule;
every comparison is exact."""
import ctypes
import json
import os
import subprocess

import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
ZETA = os.path.join(ROOT, "zeta_gb300", "_build", "zeta")


def _fixture(name):
    with open(os.path.join(HERE, "golden", name)) as f:
        return json.load(f)


def _workload(z, w):
    return z.make_positions(int(w["seed"], 16), w["n"], w["min_plies"], w["max_plies"], w["min_pieces"],
                            w["min_depth"], w["max_depth"])


@pytest.fixture
def all_promotions(zeta_device):
    z = zeta_device
    z.perft_set_promotions(True)
    try:
        yield z
    finally:
        z.perft_set_promotions(False)


def test_genmoves_all_promotions_matches_oracle(zeta_device):
    z = zeta_device
    boards, stm, _ = ol.make_positions(0xB0B, 400, min_plies=1, max_plies=160)
    special = [ol.setboard(r["fen"]) for r in _fixture("perft_promotions.json")["special"]]
    boards = np.concatenate([boards, np.stack([b for b, _ in special])])
    stm = np.concatenate([stm, np.array([s for _, s in special], np.uint8)])
    promoting = 0
    for qs in (False, True):
        lists = z.genmoves_batch(boards, stm, qs=qs, generator=0, all_promotions=True)
        for i in range(len(stm)):
            want = sorted(ol.genmoves(boards[i], stm[i], qs, all_promotions=True))
            assert sorted(lists[i].tolist()) == want, (qs, i)
            promoting += len(want) != len(ol.genmoves(boards[i], stm[i], qs))
    assert promoting >= 10
    for gen in (1, 2):
        with pytest.raises(z.ZetaError):
            z.genmoves_batch(boards[:4], stm[:4], generator=gen, all_promotions=True)


def test_promotion_setting_round_trip(zeta_device):
    z = zeta_device
    assert z.perft_get_promotions() is False
    lib = z.load_library()
    assert lib.zeta_perft_set_promotions(2) != 0
    assert z.perft_get_promotions() is False
    z.perft_set_promotions(True)
    try:
        assert z.perft_get_promotions() is True
    finally:
        z.perft_set_promotions(False)


def test_perft_bench_batch_all_promotions_at_full_size(zeta_device):
    z = zeta_device
    fx = _fixture("perft_promotions.json")
    queen = _fixture("perft_workload.json")
    boards, stm, depth = _workload(z, fx["workload"])
    want = np.array(fx["leaves"], dtype=np.uint64)
    z.perft_set_promotions(True)
    try:
        got = z.perft_batch(boards, stm, depth)
    finally:
        z.perft_set_promotions(False)
    bad = np.nonzero(got != want)[0]
    assert bad.size == 0, [(int(i), int(depth[i]), int(got[i]), int(want[i])) for i in bad[:8]]
    # back to the reference's rule: the queen-only counts again (the cached
    # launch graph must not keep the other rule)
    again = z.perft_batch(boards, stm, depth)
    assert np.array_equal(again, np.array(queen["leaves"], dtype=np.uint64))
    assert len(fx["differ_from_queen_only"]) > 0
    assert all(int(got[i]) > int(again[i]) for i in fx["differ_from_queen_only"])


def test_hand_made_promotion_positions(all_promotions):
    z = all_promotions
    for row in _fixture("perft_promotions.json")["special"]:
        b, s = ol.setboard(row["fen"])
        n = len(row["all_promotions"])
        got = z.perft_batch(np.tile(b, (n, 1)), np.full(n, s, np.uint8), np.arange(1, n + 1, dtype=np.uint8))
        assert [int(x) for x in got] == row["all_promotions"], row["fen"]


# two pawns that can take the same piece on the last rank: the bulk count
# must count both captures (a union of the two capture sets counts one)
DOUBLE_CAPTURE = ["2r4k/1P1P4/8/8/8/8/8/4K3 w - - 0 1", "4k3/8/8/8/8/8/1p1p4/2R3K1 b - - 0 1"]


def test_two_pawns_promoting_on_the_same_square(all_promotions):
    z = all_promotions
    for fen in DOUBLE_CAPTURE:
        b, s = ol.setboard(fen)
        got = z.perft_batch(np.tile(b, (4, 1)), np.full(4, s, np.uint8), np.arange(1, 5, dtype=np.uint8))
        assert [int(x) for x in got] == [ol.perft(b, s, d, all_promotions=True) for d in range(1, 5)], fen


def test_noalloc_entry_follows_the_rule(all_promotions):
    torch = pytest.importorskip("torch")
    z = all_promotions
    fx = _fixture("perft_promotions.json")
    boards, stm, depth = _workload(z, fx["workload"])
    pick = np.array([i for i in fx["differ_from_queen_only"] if depth[i] <= 4][:256])
    dev = torch.device("cuda", 0)
    db = torch.from_numpy(np.ascontiguousarray(boards[pick]).view(np.int64)).to(dev)
    ds = torch.from_numpy(np.ascontiguousarray(stm[pick])).to(dev)
    dd = torch.from_numpy(np.ascontiguousarray(depth[pick])).to(dev)
    out = torch.zeros(len(pick), dtype=torch.int64, device=dev)
    lib = z.load_library()
    rc = lib.zeta_perft_batch_noalloc(ctypes.c_void_p(db.data_ptr()), ctypes.c_void_p(ds.data_ptr()),
                                      ctypes.c_void_p(dd.data_ptr()), len(pick), ctypes.c_void_p(out.data_ptr()),
                                      ctypes.c_void_p(0))
    assert rc == 0, lib.zeta_last_error().decode()
    assert np.array_equal(out.cpu().numpy().view(np.uint64), np.array(fx["leaves"], dtype=np.uint64)[pick])


def test_zeta_binary_all_promotions_perft():
    """`zeta -u` and the `promotions` command: perft of a hand-made position
    through the six cl_* calls under both rules."""
    row = _fixture("perft_promotions.json")["special"][1]
    script = f"setboard {row['fen']}\nperft 4\npromotions queen\nperft 4\npromotions all\nperft 3\nquit\n"
    r = subprocess.run([ZETA, "-u"], input=script, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stdout + r.stderr
    counts = [int(l.split("nodecount:")[1].split(",")[0]) for l in r.stdout.splitlines() if "nodecount:" in l]
    assert counts == [row["all_promotions"][3], row["queen_only"][3], row["all_promotions"][2]], r.stdout
