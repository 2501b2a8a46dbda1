"""Build the native parts of zeta_gb300 in-tree.

* ``zeta_gb300/_build/libzeta_cuda.so`` -- the CUDA kernels and the C ABI
  of ``include/zeta_cuda.h``, compiled for sm_103a only.
* ``zeta_gb300/_build/zeta`` -- the C host (xboard / perft / selftest
  commands) linked against that library.
* ``oracle/_build/libzeta_oracle.so`` and, where the reference tree or the
  files preprocessed from it are present, ``oracle/_ref/librefzeta.so`` and
  ``oracle/_ref/zeta_refhost``: the test oracle and the reference's own
  host linked against this boundary (built by ``oracle/Makefile``'s
  ``auto`` target, which knows where the reference lives; never loaded by
  the product path).

Translation units compile in parallel; no cmake.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "zeta_gb300")
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BUILD = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + ARCH

CUDA_SOURCES = ["capi.cu", "perft.cu", "positions.cu", "peak.cu", "search.cu", "engine.cu"]
OPTIONAL_CUDA_SOURCES = ["search.cu", "mlp.cu", "noalloc.cu"]
HOST_SOURCES = ["board.c", "cudarun.c", "engine.c", "xboard.c", "main.c"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build zeta_gb300")


def _run(cmd: list[str], cwd: str | None = None) -> None:
    proc = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    inc = os.path.join(ROOT, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def build_cuda(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    sources = CUDA_SOURCES + [s for s in OPTIONAL_CUDA_SOURCES
                              if s not in CUDA_SOURCES and os.path.exists(os.path.join(CSRC, s))]
    headers = _headers()
    objs = []
    jobs = []
    for src in sources:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        if _stale(obj, [path] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", path, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    lib = os.path.join(BUILD, "libzeta_cuda.so")
    if jobs or _stale(lib, objs):
        _run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", lib] + objs)
    if verbose:
        print("built", lib)
    return lib


def build_host(verbose: bool = False) -> str | None:
    srcs = [os.path.join(HOST, s) for s in HOST_SOURCES]
    if not all(os.path.exists(s) for s in srcs):
        return None
    exe = os.path.join(BUILD, "zeta")
    deps = srcs + [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")] + _headers()
    deps.append(os.path.join(BUILD, "libzeta_cuda.so"))
    if _stale(exe, deps):
        _run(["gcc", "-O2", "-std=gnu11", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), "-o", exe] + srcs
             + ["-L", BUILD, "-lzeta_cuda", "-Wl,-rpath,$ORIGIN", "-lm"])
    if verbose:
        print("built", exe)
    return exe


def build_oracle(verbose: bool = False) -> None:
    """The oracle is test infrastructure: built so tests can load it.  The
    reference parts are optional (absent where neither the reference tree
    nor the files preprocessed from it exist)."""
    _run(["make", "-s", "-C", ORACLE])
    try:
        _run(["make", "-s", "-C", ORACLE, "auto"])
    except RuntimeError as e:
        if verbose:
            print("reference parts not built:", e, file=sys.stderr)


def build_opcount(out: str | None = None) -> str:
    """Compile and run the host op counter (csrc/opcount.cc): writes the
    algorithmic int32 operations per perft node to profiles/opcount.json."""
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, "opcount")
    _run(["g++", "-O2", "-std=c++17", "-o", exe, os.path.join(CSRC, "opcount.cc")])
    out = out or os.path.join(ROOT, "profiles", "opcount.json")
    _run([exe, out])
    return out


def build_all(verbose: bool = False) -> None:
    build_cuda(verbose)
    build_host(verbose)
    build_oracle(verbose)


if __name__ == "__main__":
    build_all(verbose=True)
