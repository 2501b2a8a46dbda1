"""Parity at the benchmark workloads' configured sizes, against fixtures the
oracle and the reference kernel produced on host cores
(tests/golden/make_workload_golden.py):

* batched perft, the whole 4096-position bench batch at its drawn depths
  3-5 (55 G leaves): every count equal to the oracle's, and 16 of them
  (depths 4 and 5) equal to the reference perft kernel's own;
* batched pure search at the configured depth 7 with the bench's table
  (1 GiB) and launch settings: the first 128 root scores equal the oracle's
  plain alpha-beta value.

Positions come from the device generator; the fixture's SHA-256 of the
positions' bytes pins them to the oracle generator's."""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _fixture(name):
    path = os.path.join(HERE, "golden", name)
    if not os.path.exists(path):
        pytest.skip(f"{name} not generated")
    return json.load(open(path))


def _sha(boards, stm, depth):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(boards, dtype="<u8").tobytes())
    h.update(np.ascontiguousarray(stm, dtype=np.uint8).tobytes())
    h.update(np.ascontiguousarray(depth, dtype=np.uint8).tobytes())
    return h.hexdigest()


def _workload(z, w):
    return z.make_positions(int(w["seed"], 16), w["n"], w["min_plies"], w["max_plies"], w["min_pieces"],
                            w["min_depth"], w["max_depth"])


def test_perft_bench_batch_equals_oracle_at_full_size(zeta_device):
    z = zeta_device
    fx = _fixture("perft_workload.json")
    boards, stm, depth = _workload(z, fx["workload"])
    assert _sha(boards, stm, depth) == fx["positions_sha256"]
    want = np.array(fx["leaves"], dtype=np.uint64)
    got = z.perft_batch(boards, stm, depth)
    bad = np.nonzero(got != want)[0]
    assert bad.size == 0, [(int(i), int(depth[i]), int(got[i]), int(want[i])) for i in bad[:8]]
    assert int(got.sum()) == fx["total_leaves"]
    # the counts the reference perft kernel itself produced
    assert len(fx["reference_subset"]) == 16
    for c in fx["reference_subset"]:
        assert int(got[c["index"]]) == c["leaves"] and int(depth[c["index"]]) == c["depth"], c


@pytest.mark.parametrize("form,workers,helpers,n", [(3, 2, 64, 1024), (1, 32, 128, 128)])
def test_search_bench_batch_depth7_equals_oracle(zeta_device, form, workers, helpers, n):
    """The bench's settings: warp-cooperative 2 workers per position with a
    helper cap of 64 over the whole 1024-position batch, and the dense form
    with 32 workers; 1 GiB table cleared first."""
    z = zeta_device
    fx = _fixture("search_workload.json")
    w = dict(fx["workload"])
    boards, stm, depth = _workload(z, w)
    assert _sha(boards, stm, depth) == fx["positions_sha256"]
    k = fx["positions"]
    z.release()
    z.init(0, 1024, 0)
    try:
        z.search_set_launch_form(form)
        z.search_set_helpers(helpers)
        z.tt_clear()
        scores, moves, nodes = z.search_batch(boards[:n], stm[:n], fx["depth"], workers)
    finally:
        z.search_set_launch_form(0)
        z.search_set_helpers(0)
        z.release()
        z.init(0, 64, 16)
    k = min(k, n)
    assert list(scores[:k]) == fx["scores"][:k]
    assert (nodes[:n] > 0).all()
