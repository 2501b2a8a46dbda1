"""The drop-in boundary with the reference's own host: the unmodified host C
of the reference (src/zeta.c, search.c, test.c, bench.c, xboard.c, io.c,
bitboard.c, bit.c, timer.c), compiled from the reference tree by
oracle/Makefile (`make refhost`) and linked with zeta_gb300/host/cudarun.c
and libzeta_cuda.so in place of its OpenCL clrun.c / clconfig.c /
clquery.c.  It runs its own selftest on the GB300 kernels and its own
iterative deepening prints the same lines as this project's host."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFHOST = os.path.join(ROOT, "oracle", "_ref", "zeta_refhost")
ZETA = os.path.join(ROOT, "zeta_gb300", "_build", "zeta")

# the reference's config.txt keys (src/io.c:533-583): one worker, a 64 MB
# TT1 and no TT2, a node rate large enough that `st 600` never binds
CONFIG = ("threadsX: 1;\nthreadsY: 1;\nnodes_per_second: 100000000;\ntt1_memory: 64;\ntt2_memory: 0;\n"
          "opencl_platform_id: 0;\nopencl_device_id: 0;\nopencl_gpugen: 0;\n")
GO_LINE = re.compile(r"^(\d+) (-?\d+) (\d+) (\d+)((?: [a-h][1-8][a-h][1-8][qrbn]?)+) *$")


def _need(path):
    if not os.path.exists(path):
        pytest.skip(f"{os.path.relpath(path, ROOT)} not built (needs the reference tree or its preprocessed host)")


def _go_lines(text):
    """(depth, score, nodes, pv) of every iterative-deepening line; the time
    column is left out."""
    out = []
    for line in text.splitlines():
        m = GO_LINE.match(line.strip())
        if m:
            out.append((int(m.group(1)), int(m.group(2)), int(m.group(4)), m.group(5).split()))
    return out


def test_refhost_links_and_starts_without_gpu():
    """The reference's host links with the boundary (no undefined symbol)
    and answers -h without touching the device."""
    _need(REFHOST)
    r = subprocess.run([REFHOST, "-h"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0
    assert "selftest" in r.stdout or "-s" in r.stdout


@pytest.mark.gpu
def test_refhost_selftest_passes_all_14(tmp_path):
    """The reference's selftest (src/test.c:36-169): its 14 perft
    known-answer positions through cl_run_perft on the GB300 kernels."""
    _need(REFHOST)
    (tmp_path / "config.txt").write_text(CONFIG)
    r = subprocess.run([REFHOST, "-s"], capture_output=True, text=True, timeout=600, cwd=tmp_path)
    assert "passed 14 from 14" in r.stdout, r.stdout[-3000:] + r.stderr[-2000:]


@pytest.mark.gpu
def test_refhost_go_lines_equal_project_host(tmp_path):
    """`new`, `st 600`, `sd 6`, `go` in console mode: the reference's
    rootsearch (src/search.c:35-223) over cudarun.c prints, depth by depth,
    the same score, cumulative node count and PV as this project's host --
    both drive zeta_engine_search with one worker from fresh tables, after
    the start-up warm-up launch at depth 0 (src/zeta.c:695)."""
    _need(REFHOST)
    _need(ZETA)
    (tmp_path / "config.txt").write_text(CONFIG)
    session = "new\nst 600\nsd 6\ngo\nquit\n"
    ref = subprocess.run([REFHOST], input=session, capture_output=True, text=True, timeout=600, cwd=tmp_path)
    ours = subprocess.run([ZETA], input=session, capture_output=True, text=True, timeout=600, cwd=tmp_path)
    assert ours.returncode == 0, ours.stderr[-2000:]
    a, b = _go_lines(ref.stdout), _go_lines(ours.stdout)
    assert [x[0] for x in b] == [1, 2, 3, 4, 5, 6], ours.stdout[-2000:]
    assert a == b, (ref.stdout[-3000:], ours.stdout[-3000:])
    # and both played the PV's first move
    moves = [l.split()[-1] for l in ref.stdout.splitlines() if l.startswith("move ")]
    assert moves and moves[-1] == b[-1][3][0]
