"""The device chess core compiled for the host (g++, no GPU), on every node
of full move trees from positions with castling, en passant, promotions,
pins and checks: the quick free-move test of the pure-search leaves agrees
with the exact legal-move count, the search kernels' generator gives the
perft generator's moves, the incremental Zobrist update equals hashing from
scratch, and the hash and the evaluation equal the oracle's."""
import os
import shutil
import subprocess

import pytest

import oracle_lib as ol

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

ROOTS = [
    ("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1", 4),
    ("r3k2r/p1ppqpb1/bn2pnp1/3PN3/1p2P3/2N2Q1p/PPPBBPPP/R3K2R w KQkq - 0 1", 3),
    ("8/2p5/3p4/KP5r/1R3p1k/8/4P1P1/8 w - - 0 1", 5),
    ("r3k2r/Pppp1ppp/1b3nbN/nP6/BBP1P3/q4N2/Pp1P2PP/R2Q1RK1 w kq - 0 1", 3),
    ("rnbq1k1r/pp1Pbppp/2p5/8/2B5/8/PPP1NnPP/RNBQK2R w KQ - 1 8", 3),
    ("4k3/8/8/8/8/8/8/4K2R w K - 0 1", 5),
    ("7k/5Q2/6K1/8/8/8/8/8 b - - 0 1", 3),
    # promotions: two pawns taking the same piece on the last rank, pushes,
    # a check blocked by a promotion, a pinned pawn
    ("2r4k/1P1P4/8/8/8/8/8/4K3 w - - 0 1", 3),
    ("4k3/8/8/8/8/8/1p1p4/2R3K1 b - - 0 1", 3),
    ("4k3/1P4P1/8/8/8/8/1p4p1/4K3 w - - 0 1", 4),
    ("K6r/2P5/8/8/8/8/8/3k4 w - - 0 1", 4),
    ("8/8/8/8/8/k7/1p6/2B4K b - - 0 1", 4),
]


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("host") / "legal_test_check")
    obj = exe + "_oracle.o"
    subprocess.run(["gcc", "-O2", "-std=c11", "-c", "-o", obj, os.path.join(ROOT, "oracle", "zeta_oracle.c")],
                   check=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "host", "legal_test_check.cc"), obj],
                   check=True)
    return exe


def _arg(board, stm, depth):
    return ":".join(str(int(x)) for x in board[:5]) + f":{int(stm)}:{depth}"


def test_leaf_test_generators_and_incremental_hash_agree(checker):
    args = []
    for fen, depth in ROOTS:
        b, s = ol.setboard(fen)
        args.append(_arg(b, s, depth))
    boards, stm, _ = ol.make_positions(0x4A13, 24, min_plies=1, max_plies=200, min_pieces=0, min_depth=0,
                                       max_depth=0)
    args += [_arg(boards[i], stm[i], 2) for i in range(len(stm))]
    r = subprocess.run([checker] + args, capture_output=True, text=True, timeout=600)
    last = r.stdout.strip().splitlines()[-1]
    assert r.returncode == 0, r.stdout[-2000:]
    nodes = int(last.split(":")[1].split()[0])
    quick = int(last.split(",")[1].split()[0])
    assert nodes > 1_000_000 and quick > nodes // 2, last
