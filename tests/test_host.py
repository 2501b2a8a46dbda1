"""The C host: its board layer against the oracle (CPU), and the zeta
binary's selftest and xboard session on the GPU."""
import os
import subprocess

import numpy as np
import pytest

import oracle_lib as ol

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "zeta_gb300", "host")
ZETA = os.path.join(ROOT, "zeta_gb300", "_build", "zeta")

HARNESS = r"""
#include <stdio.h>
#include "board.h"
int main(void) {
  char fen[512];
  while (fgets(fen, sizeof fen, stdin)) {
    Bitboard b[7]; int stm, full;
    int ok = board_setfen(b, &stm, &full, fen);
    char out[256]; board_getfen(b, stm, full, out, sizeof out);
    printf("%d %d", ok, stm);
    for (int i = 0; i < 7; i++) printf(" %llx", (unsigned long long)b[i]);
    printf(" %llx|%s\n", (unsigned long long)board_hash(b, stm), out);
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    d = tmp_path_factory.mktemp("host")
    src = d / "h.c"
    src.write_text(HARNESS)
    exe = d / "h"
    subprocess.run(["gcc", "-O1", "-std=gnu11", "-I", HOST, "-o", str(exe), str(src), os.path.join(HOST, "board.c")],
                   check=True)
    return str(exe)


FENS = ["rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1",
        "r3k2r/p1ppqpb1/bn2pnp1/3PN3/1p2P3/2N2Q1p/PPPBBPPP/R3K2R w KQkq - 0 1",
        "8/2p5/3p4/KP5r/1R3p1k/8/4P1P1/8 w - - 0 1",
        "r4rk1/1pp1qppp/p1np1n2/2b1p1B1/2B1P1b1/P1NP1N2/1PP1QPPP/R4RK1 w - - 0 10",
        "rnbqkbnr/ppp1pppp/8/3pP3/8/8/PPPP1PPP/RNBQKBNR b Kq d6 4 3",
        "4k3/8/8/8/8/8/8/4K2R w K - 0 1"]


def test_host_board_layer_matches_oracle(harness):
    out = subprocess.run([harness], input="\n".join(FENS) + "\n", capture_output=True, text=True, check=True).stdout
    for fen, line in zip(FENS, out.strip().splitlines()):
        head, fen_out = line.split("|")
        f = head.split()
        b, stm = ol.setboard(fen)
        assert int(f[0]) == 1 and int(f[1]) == stm
        assert [int(x, 16) for x in f[2:9]] == [int(x) for x in b]
        assert int(f[9], 16) == ol.computehash(b, stm)
        # the FEN the host writes sets the same board again
        b2, s2 = ol.setboard(fen_out)
        assert [int(x) for x in b2[:4]] == [int(x) for x in b[:4]] and s2 == stm


MALFORMED = ["", "garbage", "8/8/8/8/8/8/8/8 w - - 0 1", "k7/8/8/8/8/8/8/7K w - e 0 1",
             "k7/8/8/8/8/8/8/7K w - z9 0 1", "k7/8/8/8/8/8/8/7K w - e9 0 1",
             "rnbqkbnr/pppppppp/99/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1", "/" * 40 + " w",
             "K" * 300 + " b", "kK" * 40, "k7/8/8/8/8/8/8/7K x QQQQQQQQQQQQQQQQQQQQ abcdefghijklmnop 99999999999 -1",
             "8/8/8/8/8/8/8/8/8/8/8/8/k6K w - - 0 1", "x" * 2000]


def test_host_board_layer_survives_malformed_fens(tmp_path):
    """Malformed FEN lines (no kings, rank overflow, odd en-passant fields,
    over-long fields and lines) under AddressSanitizer and
    UndefinedBehaviorSanitizer: no invalid access, and a board without
    exactly one king per side is refused."""
    src = tmp_path / "h.c"
    src.write_text(HARNESS)
    exe = tmp_path / "h_san"
    r = subprocess.run(["gcc", "-O1", "-g", "-std=gnu11", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
                        "-I", HOST, "-o", str(exe), str(src), os.path.join(HOST, "board.c")], capture_output=True)
    if r.returncode != 0:
        pytest.skip("sanitizer runtime not available: " + r.stderr.decode(errors="replace")[-200:])
    out = subprocess.run([str(exe)], input="\n".join(MALFORMED) + "\n", capture_output=True, text=True,
                         timeout=60)
    assert out.returncode == 0, out.stderr[-2000:]
    for line in out.stdout.strip().splitlines():
        f = line.split("|")[0].split()
        kings = int(f[3], 16) & int(f[4], 16) & ~int(f[5], 16)
        black = int(f[2], 16)
        one_each = bin(kings & black).count("1") == 1 and bin(kings & ~black).count("1") == 1
        assert int(f[0]) == int(one_each), line


MOVE_HARNESS = r"""
#include <stdio.h>
#include <string.h>
#include "board.h"
int main(void) {
  char line[256];
  while (fgets(line, sizeof line, stdin)) {
    line[strcspn(line, "\n")] = 0;
    printf("%d\n", move_text_ok(line) ? 1 : 0);
  }
  return 0;
}
"""

MOVE_TEXT = {"e2e4": 1, "a7a8q": 1, "h2h1N": 1, "g1f3": 1, "e2e4x": 0, "e2e": 0, "": 0, "e9e4": 0, "i2e4": 0,
             "e2e4qq": 0, "E2E4": 0, "e0e1": 0, "a7a8k": 0, "x" * 200: 0, "e2-e4": 0}


def test_host_move_text_check(tmp_path):
    """Coordinate move text the xboard loop accepts before it asks the
    device for the position's legal moves: squares a-h / 1-8 and an
    optional q, r, b or n; everything else is refused, under the
    sanitizers."""
    src = tmp_path / "m.c"
    src.write_text(MOVE_HARNESS)
    exe = tmp_path / "m_san"
    r = subprocess.run(["gcc", "-O1", "-g", "-std=gnu11", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
                        "-I", HOST, "-o", str(exe), str(src), os.path.join(HOST, "board.c")], capture_output=True)
    if r.returncode != 0:
        pytest.skip("sanitizer runtime not available: " + r.stderr.decode(errors="replace")[-200:])
    texts = list(MOVE_TEXT)
    out = subprocess.run([str(exe)], input="\n".join(texts) + "\n", capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr[-2000:]
    assert [int(x) for x in out.stdout.split()] == [MOVE_TEXT[t] for t in texts]


CONFIG_HARNESS = r"""
#include <inttypes.h>
#include <stdio.h>
#include "engine.h"
int main(int argc, char **argv) {
  if (!clrun_write_config(argv[1], 384, 26000000, 2048, 64, 3, "a test device")) return 2;
  if (!read_config(argv[1])) return 3;
  printf("%" PRIu64 " %" PRIu64 " %" PRIi64 " %" PRIu64 " %" PRIu64 " %" PRIu64 " %d\n", threadsX, totalWorkUnits,
         nodes_per_second, MaxNodes, tt1_memory, tt2_memory, opencl_device_id);
  return 0;
}
"""


def test_config_file_round_trip(tmp_path):
    """What the tuner (cl_guess_config) writes, in the reference's config.txt
    key format, is what the host's read_config applies at start-up:
    workers, node rate (and the node budget from it), table sizes, device."""
    lib = os.path.join(ROOT, "zeta_gb300", "_build")
    if not os.path.exists(os.path.join(lib, "libzeta_cuda.so")):
        pytest.skip("libzeta_cuda.so not built")
    src = tmp_path / "cfg.c"
    src.write_text(CONFIG_HARNESS)
    exe = tmp_path / "cfg"
    subprocess.run(["gcc", "-O1", "-std=gnu11", "-I", HOST, "-I", os.path.join(ROOT, "include"), "-o", str(exe),
                    str(src), os.path.join(HOST, "cudarun.c"), os.path.join(HOST, "engine.c"),
                    os.path.join(HOST, "board.c"), "-L", lib, "-lzeta_cuda", "-Wl,-rpath," + lib, "-lm"], check=True)
    cfg = tmp_path / "config.txt"
    r = subprocess.run([str(exe), str(cfg)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == ["384", "384", "26000000", "26000000", "2048", "64", "3"]
    text = cfg.read_text()
    for key in ("threadsX:", "threadsY:", "nodes_per_second:", "tt1_memory:", "tt2_memory:", "opencl_device_id:"):
        assert key in text


def test_zeta_binary_help_runs_without_gpu():
    if not os.path.exists(ZETA):
        pytest.skip("host binary not built")
    r = subprocess.run([ZETA, "--help"], capture_output=True, text=True, timeout=30)
    assert r.returncode == 0 and "--selftest" in r.stdout


@pytest.mark.gpu
def test_zeta_selftest_passes_all_14():
    r = subprocess.run([ZETA, "-s"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "passed 14 from 14" in r.stdout


@pytest.mark.gpu
def test_zeta_go_prints_the_reference_search():
    """`go` through the six cl_* calls: every iterative-deepening line
    (depth, score, cumulative nodes, PV) equals the reference kernel's own
    search with the host's default tables (256 MB TT1, no TT2)."""
    if ol.reference() is None:
        pytest.skip("reference kernels (oracle/_ref) not built")
    r = subprocess.run([ZETA], input="new\nst 600\nsd 6\ngo\nquit\n", capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [l.split() for l in r.stdout.splitlines() if l[:1].isdigit()]
    assert [int(f[0]) for f in lines] == [1, 2, 3, 4, 5, 6]
    b, stm = ol.setboard("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    ref = ol.RefSearch(1 << 24, 0)
    total = 0
    for f in lines:
        pv, cnt = ref.run(b, stm, int(f[0]))
        total += int(cnt[0, 1])
        assert int(f[1]) == int(np.int32(pv[0])) and int(f[3]) == total
        assert f[4:] == [ol.move2can(int(m)) for m in pv[1:1 + int(f[0])] if m]


@pytest.mark.gpu
def test_zeta_st_one_second_moves_in_time(tmp_path):
    """Time control (src/xboard.c:426-438, src/search.c:194-198): after
    `st 1` the engine answers `go` with a legal move within about a second,
    without a depth limit, from the default configuration (one worker)."""
    import time
    p = subprocess.Popen([ZETA], stdin=subprocess.PIPE, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                         cwd=tmp_path, bufsize=1)
    try:
        p.stdin.write("xboard\nprotover 2\nnew\nst 1\nping 7\n")
        p.stdin.flush()
        while "pong 7" not in p.stdout.readline():
            pass
        t0 = time.perf_counter()
        p.stdin.write("go\n")
        p.stdin.flush()
        line = p.stdout.readline()
        while line and not line.startswith("move "):
            line = p.stdout.readline()
        dt = time.perf_counter() - t0
        p.stdin.write("quit\n")
        p.stdin.flush()
    finally:
        p.wait(timeout=60)
    assert line.startswith("move "), line
    assert dt < 1.5, f"st 1 took {dt:.2f} s"
    b, s = ol.setboard("rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1")
    assert line.split()[1] in {ol.move2can(m) for m in ol.genmoves(b, s)}


@pytest.mark.gpu
def test_zeta_benchfile_sweeps_workers_over_a_position_list(tmp_path):
    """benchfile (the harness of the reference's benchkaufmann /
    benchhyatt24, src/xboard.c:975-1428): a worker sweep per position, one
    results.txt table each, then the table of the summed times."""
    fens = tmp_path / "positions.epd"
    fens.write_text("r3k2r/p1ppqpb1/bn2pnp1/3PN3/1p2P3/2N2Q1p/PPPBBPPP/R3K2R w KQkq -\n"
                    "# a comment line\n"
                    "8/2p5/3p4/KP5r/1R3p1k/8/4P1P1/8 w - -\n")
    r = subprocess.run([ZETA], input=f"sd 4\nbenchfile {fens} 2\nquit\n", capture_output=True, text=True,
                       timeout=600, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    out = r.stdout
    assert "### setting up board 2: ###" in out and "### all 2 positions: ###" in out
    rows = [l.split() for l in out.splitlines() if l.startswith("### 1\t") or l.startswith("### 2\t")]
    assert len(rows) == 6  # workers 1 and 2, for two positions and the sum
    total = out.split("### all 2 positions: ###")[1]
    assert total.count("\n### 1\t") == 1 and total.count("\n### 2\t") == 1


@pytest.mark.gpu
def test_zeta_xboard_session_plays_a_legal_move():
    session = "xboard\nprotover 2\nnew\nsd 4\nusermove e2e4\nquit\n"
    r = subprocess.run([ZETA], input=session, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    moves = [l.split()[1] for l in r.stdout.splitlines() if l.startswith("move ")]
    assert len(moves) == 1
    b, s = ol.setboard("rnbqkbnr/pppppppp/8/8/4P3/8/PPPP1PPP/RNBQKBNR b KQkq - 0 1")
    legal = {ol.move2can(m) for m in ol.genmoves(b, s)}
    assert moves[0] in legal


@pytest.mark.gpu
def test_zeta_refuses_illegal_and_malformed_user_moves():
    """`usermove` plays only a legal move of the position (the device's
    generator lists them, under-promotions included): malformed text and
    illegal moves are answered with "Illegal move" and leave the game as
    it was; an under-promotion is played as the piece named."""
    session = ("new\nforce\nusermove e2e5\nusermove e2\nusermove e7e5\nusermove e2e4\nusermove e7e5\n"
               "setboard 4k3/1P6/8/8/8/8/8/4K3 w - - 0 1\nusermove b7b8n\nprint\nquit\n")
    r = subprocess.run([ZETA], input=session, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    illegal = [l.split(":", 1)[1].strip() for l in r.stdout.splitlines() if l.startswith("Illegal move:")]
    # e7e5 is illegal the first time (white to move), legal after e2e4
    assert illegal == ["e2e5", "e2", "e7e5"], r.stdout
    fen = [l[2:] for l in r.stdout.splitlines() if l.startswith("# ") and "/" in l][-1]
    b, s = ol.setboard(fen)
    want, ws = ol.setboard("1N2k3/8/8/8/8/8/8/4K3 b - - 0 1")
    assert [int(x) for x in b[:4]] == [int(x) for x in want[:4]] and s == ws, fen
