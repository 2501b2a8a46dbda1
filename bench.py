"""Benchmark of the Zeta device path on GB300.

Default workload (one "step"): batched perft over 4096 seeded random
playout positions (10-60 plies from the initial position, terminal
positions discarded) at depths drawn uniformly from 3-5, in one persistent
work-stealing launch sequence.  Metric: perft leaves per second, bit-exact
(every step's counts are checked against the first step's).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's own perft kernel (src/zetaperft.cl,
compiled for the host from the unmodified source under a work-group
emulator, oracle/_ref) on all host cores, on a bounded sample of the same
workload.  Under torchrun each rank takes its own shard of positions
(weak scaling; there is no device collective), rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "perft nodes/s (bit-exact)"
UNIT = "leaves/s"
WORKLOAD = "perft_batch"
L2_FLUSH_BYTES = 256 << 20

# Algorithmic 32-bit integer operations per node of the perft kernel
# (u64 and/or/xor/not/add/sub/compare = 2, shift = 2 constant / 4 variable,
# popc/ctz = 2), counted by zeta_gb300/csrc/opcount.cc on the initial
# position's depth-5 tree with the kernel's own code; fixed, never retuned.
OPS_PER_COUNTED_NODE = None  # filled from profiles/opcount.json when present
OPS_PER_INTERIOR_NODE = None


def _opcounts(tree: str = "startpos_d5"):
    """Algorithmic int32 operations per bulk-counted and per interior perft
    node, counted once on the perft generator's own code
    (zeta_gb300/csrc/opcount.cc): over the initial position's depth-5 tree
    (the fixed denominator) or over the 64-position workload sample."""
    path = os.path.join(ROOT, "profiles", "opcount.json")
    if os.path.exists(path):
        d = json.load(open(path))[tree]
        return d["ops_per_counted_node"], d["ops_per_interior_node"]
    return None, None


def _node_roofline(z, nodes_per_s: float, key: str, kernel: str):
    """int32-ALU roofline of a search kernel: nodes/s x algorithmic ops per
    node (profiles/opcount.json) against the measured integer peak."""
    path = os.path.join(ROOT, "profiles", "opcount.json")
    if not os.path.exists(path):
        return None
    ops = json.load(open(path)).get(key)
    try:
        peak = z.int_peak_tops()
    except Exception:  # noqa: BLE001 -- the microbenchmark is optional
        return None
    if not ops or not peak:
        return None
    achieved = nodes_per_s * ops / 1e12
    return {"bound": "int32-alu", "achieved": round(achieved, 4), "peak": round(peak, 3), "unit": "Tops/s",
            "frac": round(achieved / peak, 4), "traffic": None, "ops_per_node": ops, "kernel": kernel,
            "peak_source": "measured: int32 LOP3/SHF/IADD3 microbenchmark (zeta_int_peak)"}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        return json.load(open(path))
    return {}


def shard_seed(seed: int, rank: int) -> int:
    """The seed of rank `rank`'s shard of a workload: ranks are replicas
    that each take their own positions (weak scaling)."""
    return seed + 0x1000003 * rank


def reduce_over_ranks(seconds: float, units: float, device) -> tuple[float, float]:
    """The job's timing across replicas: the slowest rank's seconds and the
    units all ranks processed (an all-reduce on the host's process group;
    the search path itself has no collective)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(c)
    return float(t.item()), float(c.item())


def workload_arrays(z, rank: int, n: int = 0):
    w = dict(z.WORKLOADS[WORKLOAD])
    return z.make_positions(shard_seed(w["seed"], rank), n or w["n"], w["min_plies"], w["max_plies"],
                            w["min_pieces"], w["min_depth"], w["max_depth"])


def run_ours(args):
    import torch
    import zeta_gb300 as z

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    z.init(local, 0, 0)
    from zeta_gb300.autotune import load_tuned
    load_tuned(z)  # the autotuner's launch configuration, when recorded
    z.perft_set_promotions(args.all_promotions)
    info = z.device_info()
    boards, stm, depth = workload_arrays(z, rank, args.n)
    n = len(depth)
    dev = torch.device("cuda", local)
    d_boards = torch.from_numpy(boards.view(np.int64)).to(dev)
    d_stm = torch.from_numpy(stm).to(dev)
    d_depth = torch.from_numpy(depth).to(dev)
    d_leaves = torch.zeros(n, dtype=torch.int64, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    # a non-default stream: the library captures its launch sequence on it
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream

    def step():
        z.perft_batch_device(d_boards.data_ptr(), d_stm.data_ptr(), d_depth.data_ptr(), n, d_leaves.data_ptr(), sp)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ref_counts = d_leaves.cpu().numpy().view(np.uint64).copy()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    kernel_ms, counted, interior = [], 0, 0
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for i in range(args.steps):
            flush.fill_(i)  # write 256 MB (> L2) between timed steps
            starts[i].record(stream)
            step()
            ends[i].record(stream)
            st = z.perft_stats()
            kernel_ms.append(st["kernel_ms"])
            counted += st["counted_nodes"]
            interior += st["interior_nodes"]
            got = d_leaves.cpu().numpy().view(np.uint64)
            if not np.array_equal(got, ref_counts):
                raise SystemExit("perft counts changed between steps")
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_s = sum(step_ms) / 1e3
    leaves_rank = int(ref_counts.sum()) * args.steps
    if world > 1:
        total_s, leaves_all = reduce_over_ranks(total_s, leaves_rank, dev)
    else:
        leaves_all = float(leaves_rank)
    value = leaves_all / total_s

    # end to end: host buffers through the public C API (H2D + launch + D2H)
    e2e_s = 0.0
    for i in range(args.steps):
        flush.fill_(i)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = z.perft_batch(boards, stm, depth)
        e2e_s += time.perf_counter() - t0
        if not np.array_equal(out, ref_counts):
            raise SystemExit("host-buffer counts differ from device-buffer counts")
    e2e_value = leaves_rank / e2e_s * (leaves_all / leaves_rank)

    if rank != 0:
        z.release()
        return
    peaks = measured_peaks()
    ops_c, ops_i = _opcounts()
    int_peak = None
    try:
        int_peak = z.int_peak_tops()
    except Exception:  # noqa: BLE001 -- the microbenchmark is optional
        int_peak = None
    kernel_avg_ms = sum(kernel_ms) / len(kernel_ms)
    roofline = None
    # the per-node operation counts are those of the queen-only kernel
    if ops_c and int_peak and not args.all_promotions:
        ops = (counted / args.steps) * ops_c + (interior / args.steps) * ops_i
        achieved = ops / (kernel_avg_ms / 1e3) / 1e12
        wc, wi = _opcounts("workload_sample")
        ops_w = (counted / args.steps) * wc + (interior / args.steps) * wi
        traffic = None
        tp = os.path.join(ROOT, "profiles", "perft_ws_traffic.json")
        if os.path.exists(tp):
            traffic = json.load(open(tp)).get("bytes_per_launch")
        roofline = {"bound": "int32-alu", "achieved": round(achieved, 3), "peak": round(int_peak, 3),
                    "unit": "Tops/s", "frac": round(achieved / int_peak, 4), "traffic": traffic,
                    "peak_source": "measured: int32 LOP3/SHF/IADD3 microbenchmark (zeta_int_peak)",
                    "kernel": "k_perft_ws",
                    "ops_per_node": {"counted": ops_c, "interior": ops_i,
                                     "source": "initial position, depth-5 tree (fixed once)"},
                    "frac_workload_sample_ops": round(ops_w / (kernel_avg_ms / 1e3) / 1e12 / int_peak, 4)}
    cpu = None if (args.no_cpu or args.all_promotions) else cpu_baseline_sample(boards, stm, depth)
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(sum(step_ms) / len(step_ms), 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded random playouts)",
        "config": perft_config(n, world, args.all_promotions),
        "leaves_per_step_per_gpu": int(ref_counts.sum()), "perft_launch": z.perft_config(),
        "e2e": {"value": round(e2e_value, 1), "unit": UNIT, "h2d_bytes_per_step": n * 58,
                "d2h_bytes_per_step": n * 8},
        "gpu_launches": 14 * args.steps,
        "kernel_ms": round(kernel_avg_ms, 4),
        "nodes": {"counted_per_step": counted // args.steps, "interior_per_step": interior // args.steps},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
        "device": {"sms": info["sms"], "cc": list(info["cc"]), "hbm_gbs_measured": peaks.get("hbm_gbs")},
    }
    if not args.no_search:
        z.release()
        line["search_batch"] = search_batch_block(z, local, rank, args)
        line["learned_ab"] = learned_ab_block(z, local, rank, args)
    print(json.dumps(line), flush=True)
    z.release()


def _search_setting():
    """(launch form, ABDADA workers per position, helper cap) of the default
    line's batched search: the autotuner's record (python -m
    zeta_gb300.autotune search), else warp-cooperative, 2 workers, helpers
    up to 64 per position.  The table stays at the configured 1 GiB."""
    from zeta_gb300.autotune import load_search_tuned
    t = load_search_tuned()
    return t["form"], t["workers"], t["helpers"]


def _search_arrays(z, rank, n):
    w = dict(z.WORKLOADS["search_batch"])
    return z.make_positions(shard_seed(w["seed"], rank), n or w["n"], w["min_plies"], w["max_plies"],
                            w["min_pieces"], 0, 0)[:2]


def oracle_search_sample(boards, stm, depth: int, budget_s: float = 15.0):
    """The oracle's plain alpha-beta (oracle/zeta_oracle.c, ordered moves,
    the same root values) on the host cores, a bounded sample of the
    workload: positions/s, labelled as the oracle, not the reference (the
    reference has no pure fixed-depth search)."""
    from concurrent.futures import ThreadPoolExecutor
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as ol
    cores = os.cpu_count() or 1
    k = min(len(stm), cores)
    t0 = time.perf_counter()
    with ThreadPoolExecutor(cores) as ex:  # the ctypes calls release the GIL
        vals = list(ex.map(lambda i: ol.alphabeta_ordered(boards[i], int(stm[i]), depth)[0], range(k)))
    dt = time.perf_counter() - t0
    if dt < budget_s / 4 and 2 * k <= len(stm):
        k2 = min(len(stm), int(k * min(8.0, budget_s / max(dt, 1e-3))))
        t0 = time.perf_counter()
        with ThreadPoolExecutor(cores) as ex:
            vals = list(ex.map(lambda i: ol.alphabeta_ordered(boards[i], int(stm[i]), depth)[0], range(k2)))
        dt, k = time.perf_counter() - t0, k2
    return {"value": round(k / dt, 3), "unit": "positions/s", "cores": cores, "kind": "port",
            "label": "oracle, not reference",
            "sample": f"oracle plain alpha-beta (ordered moves, no table) on {cores} host threads, first {k} "
                      f"workload positions at depth {depth} in {dt:.1f}s"}, vals


def search_batch_block(z, local, rank, args):
    """Batched pure search (1024 playout positions, depth 7, 1 GiB table
    cleared every step), device buffers, CUDA events on the launching
    stream; root scores checked against the oracle on the CPU sample."""
    import torch
    z.init(local, 1024, 0)
    boards, stm = _search_arrays(z, rank, 0)
    n, depth = len(stm), 7
    dev = torch.device("cuda", local)
    d_b = torch.from_numpy(boards.view(np.int64)).to(dev)
    d_s = torch.from_numpy(stm).to(dev)
    d_sc = torch.zeros(n, dtype=torch.int32, device=dev)
    d_mv = torch.zeros(n, dtype=torch.int32, device=dev)
    d_nd = torch.zeros(n, dtype=torch.int64, device=dev)
    stream = torch.cuda.Stream(dev)
    s_form, s_workers, s_helpers = _search_setting()
    z.search_set_launch_form(s_form)
    z.search_set_helpers(s_helpers)

    def step():
        z.tt_clear()
        z.search_batch_device(d_b.data_ptr(), d_s.data_ptr(), n, depth, s_workers, d_sc.data_ptr(),
                              d_mv.data_ptr(), d_nd.data_ptr(), stream.cuda_stream)

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    steps = 3
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    kms, nodes, probes, stores = [], 0, 0, 0
    with ClockSampler(local) as clocks:
        for a, b in ev:
            a.record(stream)
            step()
            b.record(stream)
            kms.append(z.search_last_ms())
            pr, sto = z.search_last_table_ops()
            probes += pr
            stores += sto
            nodes += int(d_nd.sum().item())
        torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in ev]
    scores = d_sc.cpu().numpy().copy()
    z.search_set_launch_form(0)
    z.search_set_helpers(0)
    total_s = sum(ms) / 1e3
    nps = nodes / total_s
    roofline = _node_roofline(z, nps, "ops_per_search_node", "k_search_warp" if s_form == 3 else "k_search_pure")
    # the table's traffic, counted on the device: one 32-byte sector per
    # probe or store, against the measured HBM copy bandwidth
    tt_bytes = 32 * (probes + stores) / steps
    hbm = measured_peaks().get("hbm_gbs")
    tt_gbs = tt_bytes / (sum(kms) / len(kms) / 1e3) / 1e9
    table = {"probes_per_step": probes // steps, "stores_per_step": stores // steps,
             "bytes_per_step": int(tt_bytes), "gbs": round(tt_gbs, 2), "hbm_peak_gbs": hbm,
             "frac_of_hbm": round(tt_gbs / hbm, 4) if hbm else None,
             "rule": "32 B sector per 16-byte entry probed or stored, counted on the device"}
    z.release()
    cpu, vals = (None, None) if args.no_cpu else oracle_search_sample(boards, stm, depth)
    if vals is not None and list(scores[:len(vals)]) != [int(v) for v in vals]:
        raise SystemExit("batched search root scores differ from the oracle's")
    return {
        "metric": f"batched search positions/s (fixed depth {depth}, root score = plain negamax)",
        "value": round(n * steps / total_s, 2), "unit": "positions/s", "steps": steps, "warmup": 3,
        "ms_per_step": round(sum(ms) / steps, 3), "kernel_ms": round(sum(kms) / len(kms), 3),
        "config": {"workload": f"search_batch: {n} playouts of 20-40 plies, >=20 pieces, depth {depth}",
                   "form": {1: "dense", 2: "sparse", 3: "warp-cooperative"}.get(s_form, "automatic"),
                   "workers_per_position": s_workers,
                   "helper_cap": s_helpers, "tt": "1 GiB, 16-byte entries, cleared every step",
                   "l2": "the 1 GiB table and 2.4 G node visits per step exceed L2"},
        "nodes_per_s": round(nps, 1), "nodes_per_step": nodes // steps,
        "roofline": roofline, "table_traffic": table,
        "oracle_cpu": cpu, "scores_checked_against_oracle": 0 if vals is None else len(vals),
        "clocks": clocks.summary(), "gpu_launches": steps * 3,
    }


def learned_ab_block(z, local, rank, args):
    """Learned vs plain move ordering: iterative deepening 1..8 of the
    search workload with the hand-written ordering and with the BF16
    network, interleaved pairs from cleared tables; root scores must be
    identical, time to depth and nodes are compared."""
    from zeta_gb300 import learn
    z.init(local, 1024, 0)
    boards, stm = _search_arrays(z, rank, args.ab_n or 512)
    model = args.ab_model or learn.MODEL
    if not learn.load(z, model):
        z.release()
        return {"unavailable": f"no trained network ({os.path.relpath(model, ROOT)})", "gpu_launches": 0}
    depth, pairs = args.ab_depth, args.ab_pairs
    _, s_workers, s_helpers = _search_setting()
    z.search_set_helpers(s_helpers)
    runs = {0: [], 1: []}
    identical = True
    try:
        with ClockSampler(local) as clocks:
            for _ in range(pairs):
                for o in (0, 1):
                    z.tt_clear()
                    sc, mv, nodes, ms, ms_s, ms_n = z.search_id(boards, stm, depth, s_workers, o)
                    runs[o].append({"ms": ms, "nodes": int(nodes.sum()), "ms_net": ms_n, "scores": sc})
                identical = identical and np.array_equal(runs[0][-1]["scores"], runs[1][-1]["scores"])
    finally:
        z.search_set_helpers(0)
        z.release()

    def med(o, k):
        return statistics.median(r[k] for r in runs[o])

    ratio_t = [b["ms"] / a["ms"] for a, b in zip(runs[0], runs[1])]
    ratio_n = [b["nodes"] / a["nodes"] for a, b in zip(runs[0], runs[1])]
    return {
        "metric": f"time to depth {depth}, learned (BF16 network) vs plain ordering, same root scores",
        "config": {"workload": f"search_batch: {len(stm)} playouts, iterative deepening 1..{depth}",
                   "model": os.path.relpath(model, ROOT),
                   "form": "automatic (warp-cooperative)", "workers_per_position": s_workers,
                   "helper_cap": s_helpers, "pairs": pairs, "order": "plain then learned, interleaved"},
        "plain": {"ms_median": round(med(0, "ms"), 1), "ms_runs": [round(r["ms"], 1) for r in runs[0]],
                  "nodes_median": med(0, "nodes"), "nodes_runs": [r["nodes"] for r in runs[0]]},
        "learned_bf16": {"ms_median": round(med(1, "ms"), 1), "ms_runs": [round(r["ms"], 1) for r in runs[1]],
                         "nodes_median": med(1, "nodes"), "nodes_runs": [r["nodes"] for r in runs[1]],
                         "network_ms_median": round(med(1, "ms_net"), 2)},
        "time_ratio_median": round(statistics.median(ratio_t), 4),
        "time_ratio_range": [round(min(ratio_t), 4), round(max(ratio_t), 4)],
        "nodes_ratio_median": round(statistics.median(ratio_n), 4),
        "nodes_ratio_range": [round(min(ratio_n), 4), round(max(ratio_n), 4)],
        "scores_identical": bool(identical), "clocks": clocks.summary(),
        "gpu_launches": pairs * 2 * depth + pairs * (depth - 1) * 4,
    }


def run_learned_ab(args):
    """The learned-ordering A/B alone, by default on the whole 1024-position
    search workload at depth 8 (the configured size)."""
    import torch
    import zeta_gb300 as z
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    args.ab_n = args.ab_n or 1024
    block = learned_ab_block(z, local, rank, args)
    if rank == 0:
        print(json.dumps(dict(block, n_gpus=world, dtype="int32 search, bf16 network",
                              data="synthetic (seeded random playouts)")), flush=True)


def _ref_lib():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as ol
    if ol.reference() is None:
        return None, None
    return ol, ol.reference()


def perft_config(n: int, world: int, all_promotions: bool = False) -> dict:
    """The batched-perft workload, as both arms of the bench name it (the
    same `config` object in both lines)."""
    return {"workload": f"{WORKLOAD}: {n} seeded playouts of 10-60 plies, perft depth U[3,5]",
            "positions_per_gpu": n,
            "promotions": ("queen, rook, bishop, knight (not the reference's rule)" if all_promotions
                           else "queen only (the reference's rule)"),
            "l2": "flushed between timed GPU steps (256 MB write)", "parallelism": f"replicas x{world}"}


def reference_sample_size(cores: int) -> int:
    """Positions per sample of the reference perft kernel on the host: four
    per thread, so that every thread stays busy to the end."""
    return 4 * cores


def cpu_baseline_sample(boards, stm, depth):
    """The reference perft kernel on the host cores, on a bounded sample of
    the workload: the first 4 x threads positions at depth 3 (leaves/s does
    not depend on depth for a kernel that visits every leaf) -- the same
    sample as each step of --impl reference."""
    ol, ref = _ref_lib()
    if ref is None:
        return {"value": None, "unit": UNIT, "cores": 0, "kind": "reference",
                "sample": "reference kernels not built on this host"}
    cores = os.cpu_count() or 1
    k = min(len(depth), reference_sample_size(cores))
    d3 = np.full(k, 3, dtype=np.int32)
    t0 = time.perf_counter()
    out = ol.ref_perft_batch(boards[:k], stm[:k], d3, cores)
    dt = time.perf_counter() - t0
    leaves = int(out.sum())
    return {"value": round(leaves / dt, 1), "unit": UNIT, "cores": cores, "kind": "reference",
            "sample": f"unmodified zetaperft.cl on {cores} host threads (64-lane work-group emulator), "
                      f"first {k} workload positions at depth 3, {leaves} leaves in {dt:.1f}s"}


def run_search(args):
    """Batched fixed-depth pure search: 1024 seeded playout positions (20-40
    plies, >= 20 pieces) at depth 7, ABDADA workers per position, 1 GiB
    transposition table cleared at the start of every step (part of the
    timed work).  Metric: positions per second."""
    import torch
    import zeta_gb300 as z
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    z.init(local, 1024, 0)
    w = dict(z.WORKLOADS["search_batch"])
    n = args.n or w["n"]
    boards, stm, _ = z.make_positions(shard_seed(w["seed"], rank), n, w["min_plies"], w["max_plies"],
                                      w["min_pieces"], 0, 0)
    depth = args.depth or 7
    dev = torch.device("cuda", local)
    d_b = torch.from_numpy(boards.view(np.int64)).to(dev)
    d_s = torch.from_numpy(stm).to(dev)
    d_sc = torch.zeros(n, dtype=torch.int32, device=dev)
    d_mv = torch.zeros(n, dtype=torch.int32, device=dev)
    d_nd = torch.zeros(n, dtype=torch.int64, device=dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    # (launch form, workers per position, helper cap): form 1 = dense (one
    # worker per thread), 3 = warp-cooperative (one worker per warp, the
    # lanes score the last ply); helpers let finished workers join
    # unfinished positions up to `cap` workers each (0 = no helping)
    workers_list = ([(args.form, args.workers, args.helpers)] if args.workers else
                    [(1, 32, 128), (3, 1, 16), (3, 2, 16), (3, 2, 32), (3, 2, 64), (3, 3, 32)])
    results = {}
    ref_scores = None
    names = ["auto", "dense", "sparse", "warp"]

    def measure(form, W, cap, warm, steps):
        z.search_set_launch_form(form)
        z.search_set_helpers(cap)
        for _ in range(warm):
            z.tt_clear()
            z.search_batch_device(d_b.data_ptr(), d_s.data_ptr(), n, depth, W, d_sc.data_ptr(), d_mv.data_ptr(),
                                  d_nd.data_ptr(), stream.cuda_stream)
        int(d_nd.sum().item())  # load torch's reduction kernel before the timed steps use it
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nodes = 0
        kms = []
        for _ in range(steps):
            z.tt_clear()
            z.search_batch_device(d_b.data_ptr(), d_s.data_ptr(), n, depth, W, d_sc.data_ptr(), d_mv.data_ptr(),
                                  d_nd.data_ptr(), stream.cuda_stream)
            kms.append(z.search_last_ms())
            nodes += int(d_nd.sum().item())
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / steps
        sc = d_sc.cpu().numpy().copy()
        nonlocal ref_scores
        if ref_scores is None:
            ref_scores = sc
        if not np.array_equal(sc, ref_scores):
            raise SystemExit(f"root scores changed with form {form}, {W} workers")
        return {"positions_per_s": n / dt, "ms_per_step": dt * 1e3, "kernel_ms": sum(kms) / len(kms),
                "nodes_per_s": nodes / steps / dt, "nodes_per_step": nodes // steps}

    # the sweep takes one step per setting; the best setting (or the one
    # given) is then timed over --steps steps after --warmup warm-up steps
    if len(workers_list) > 1:
        for form, W, cap in workers_list:
            key = f"{names[form]}:{W}/{cap}"
            results[key] = measure(form, W, cap, 1, 1)
            print(json.dumps({"form:workers/helper_cap": key, **results[key]}), file=sys.stderr, flush=True)
        best_w = max(results, key=lambda k: results[k]["positions_per_s"])
        form, W, cap = workers_list[list(results).index(best_w)]
    else:
        form, W, cap = workers_list[0]
        best_w = f"{names[form]}:{W}/{cap}"
    with ClockSampler(local) as clocks:
        r = measure(form, W, cap, args.warmup, args.steps)
    if rank == 0:
        print(json.dumps({
            "metric": f"batched search positions/s (fixed depth {depth}, root score = plain negamax)",
            "value": round(r["positions_per_s"], 2), "unit": "positions/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(r["ms_per_step"], 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded random playouts)",
            "config": {"workload": f"search_batch: {n} playouts of 20-40 plies, >=20 pieces, depth {depth}",
                       "form:workers_per_position/helper_cap": best_w,
                       "tt": "1 GiB, 16-byte entries, cleared every step"},
            "nodes_per_s": round(r["nodes_per_s"], 1), "nodes_per_step": r["nodes_per_step"],
            "kernel_ms": round(r["kernel_ms"], 3), "clocks": clocks.summary(),
            "sweep_single_step": {str(k): round(v["positions_per_s"], 2) for k, v in results.items()},
            "roofline": _node_roofline(z, r["nodes_per_s"], "ops_per_search_node",
                                       "k_search_warp" if best_w.startswith("warp") else "k_search_pure"),
        }), flush=True)
    z.search_set_launch_form(0)
    z.release()


def run_engine(args):
    """Full-engine search (the reference's heuristics): 256 seeded playout
    positions (20-40 plies, >= 20 pieces), iterative deepening to a depth
    with ABDADA workers per position, 8 GB TT1 + 2 GB TT2 split evenly over
    the positions; plain ordering vs the move-ordering network (BF16).
    Metric: positions per second to the depth (time-to-depth of the batch)."""
    import torch
    import zeta_gb300 as z
    from zeta_gb300 import learn
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    z.init(local, 8192, 2048)
    w = dict(z.WORKLOADS["engine"])
    n = args.n or 256
    boards, stm, _ = z.make_positions(shard_seed(w["seed"], rank), n, w["min_plies"], w["max_plies"],
                                      w["min_pieces"], 0, 0)
    depth = args.depth or 8
    workers = args.workers or 32
    have_net = learn.load(z)
    cases = [0] + ([1] if have_net else [])
    z.engine_id(boards[:32], stm[:32], min(depth, 5), workers, 0)  # warm-up (buffers, code)
    res = {}
    with ClockSampler(local) as clocks:
        for o in cases:
            sc, mv, nodes, dd, ms, ms_s, ms_n = z.engine_id(boards, stm, depth, workers, o)
            res[o] = {"scores": sc, "moves": mv, "nodes": int(nodes.sum()), "ms_total": ms, "ms_search": ms_s,
                      "ms_network": ms_n, "depth_min": int(dd.min())}
            print(json.dumps({"ordering": o, "nodes": res[o]["nodes"], "ms_total": round(ms, 2),
                              "ms_network": round(ms_n, 2), "depth_min": res[o]["depth_min"]}), file=sys.stderr,
                  flush=True)
    p = res[0]
    line = {
        "metric": f"full-engine search positions/s to depth {depth} (reference heuristics)",
        "value": round(n / (p["ms_total"] / 1e3), 3), "unit": "positions/s", "n_gpus": world, "steps": 1,
        "warmup": 1, "ms_per_step": round(p["ms_total"], 2), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded random playouts)",
        "config": {"workload": f"engine: {n} playouts of 20-40 plies, >=20 pieces, iterative deepening 1..{depth}",
                   "workers_per_position": workers, "tt": "8 GB TT1 + 2 GB TT2, 1/n per position"},
        "nodes_per_s": round(p["nodes"] / (p["ms_total"] / 1e3), 1), "nodes": p["nodes"],
        "clocks": clocks.summary(),
        "roofline": _node_roofline(z, p["nodes"] / (p["ms_total"] / 1e3), "ops_per_engine_node", "k_engine"),
    }
    if 1 in res:
        l1 = res[1]
        line["learned_bf16"] = {
            "ms_total": round(l1["ms_total"], 2), "ms_network": round(l1["ms_network"], 2), "nodes": l1["nodes"],
            "time_to_depth_ratio": round(l1["ms_total"] / p["ms_total"], 4),
            "score_agreement": round(float((l1["scores"] == p["scores"]).mean()), 4),
            "best_move_agreement": round(float((l1["moves"] == p["moves"]).mean()), 4)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    z.release()


def run_smp(args):
    """The reference's own published search benchmark (results.txt,
    `benchsmp`): the full engine's iterative deepening from the initial
    position to depth 12, one position, fresh tables, with a growing number
    of workers.  Metric: time to depth (s, lower is better); the best
    published figure is 4.871 s (Titan RTX, 128 workers, results.txt:37)."""
    import torch
    import zeta_gb300 as z
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    z.init(local, args.tt1_mb, args.tt2_mb)
    z.engine_set_helper_depth(args.deep_every)
    depth = args.depth or 12
    wlist = [args.workers] if args.workers else [int(x) for x in args.smp_workers.split(",")]
    b = z.STARTPOS

    def run(W):
        z.tt_clear()
        nodes, t0, launches, sc, pv = 0, time.perf_counter(), 0, 0, None
        for d in range(1, depth + 1):
            pv, cnt = z.engine_search(b, 0, d, W)
            launches += 1
            nodes += int(cnt[:, 1].sum())
            sc = int(np.int32(pv[0]))
            if abs(sc) >= 30000 and d >= 32000 - abs(sc):
                break  # mate in n: no deeper iteration changes it
        dt = time.perf_counter() - t0
        return {"workers": W, "seconds": round(dt, 3), "nps": round(nodes / dt, 1), "nodes": nodes, "score": sc,
                "move": int(pv[1]), "launches": launches}

    rows = []
    with ClockSampler(local) as clocks:
        # the worker sweep (benchsmp's table); multi-worker searches vary run
        # to run, so each count is run three times and ranked by its median
        for W in wlist:
            trio = sorted((run(W) for _ in range(3 if len(wlist) > 1 else 1)), key=lambda r: r["seconds"])
            rows.append(dict(trio[len(trio) // 2], runs_s=[r["seconds"] for r in trio]))
            print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
        # then the best count again, --steps runs, reported by their median
        w_best = min(rows, key=lambda r: r["seconds"])["workers"]
        reps = [run(w_best) for _ in range(max(1, args.steps))]
        for r in reps:
            print(json.dumps(dict(r, repeat=True)), file=sys.stderr, flush=True)
    reps.sort(key=lambda r: r["seconds"])
    best = reps[len(reps) // 2]  # the median run
    if rank == 0:
        print(json.dumps({
            "metric": f"full-engine time to depth {depth} from the initial position (reference benchsmp)",
            "value": best["seconds"], "unit": "s", "n_gpus": world, "steps": len(reps), "warmup": 0,
            "ms_per_step": round(best["seconds"] * 1e3, 1), "higher_is_better": False, "scaling": "replicas",
            "vs_baseline": round(best["seconds"] / 4.871, 4) if depth == 12 else None,
            "baseline": "4.871 s: Titan RTX, 128 work-groups, version 099k (results.txt:37)",
            "dtype": "int32", "data": "the initial position",
            "config": {"workload": f"startpos iterative deepening 1..{depth}, {args.tt1_mb} MB TT1 + {args.tt2_mb} MB "
                                   "TT2, fresh tables",
                       "workers": best["workers"], "statistic": f"median of {len(reps)} runs",
                       "helper_depth": (f"every {args.deep_every}th helper one ply deeper" if args.deep_every
                                        else "all workers at the iteration depth (the reference's)"),
                       "runs_s": [r["seconds"] for r in reps]},
            "nodes_per_s": best["nps"],
            "e2e": {"value": best["seconds"], "unit": "s", "h2d_bytes_per_step": 58 * best["launches"],
                    "d2h_bytes_per_step": (256 + 512 * best["workers"]) * best["launches"]},
            "gpu_launches": best["launches"], "clocks": clocks.summary(), "scaling_table": rows,
        }), flush=True)
    z.release()


GEMM_SHAPES = (
    # (M, N, K): the move-ordering network's layers at a 65536-position batch
    (65536, 512, 768),   # forward layer 1 (768 one-hot -> 512)
    (65536, 256, 512),   # forward layer 2
    (65536, 128, 256),   # head (q_from, q_to)
    (768, 512, 65536),   # weight gradient of layer 1 (K = positions)
    (8192, 8192, 8192),  # square, the shape of the measured bf16 peak
)


def run_gemm(args):
    """The tensor-core GEMM (zeta_gemm_tc, tcgen05.mma, FP32 accumulation)
    on the network's shapes, BF16 and FP8, next to torch.matmul (cuBLAS) on
    the same BF16 operands.  Metric: TFLOP/s (2*M*N*K per product)."""
    import torch
    import zeta_gb300 as z
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    z.init(local, 0, 0)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    g = torch.Generator(device=dev).manual_seed(7)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    peaks = measured_peaks()
    rows = []
    pick = [int(x) for x in args.gemm_shapes.split(",")] if args.gemm_shapes else range(len(GEMM_SHAPES))
    for (M, N, K) in [GEMM_SHAPES[i] for i in pick]:
        A = (torch.rand(M, K, device=dev, generator=g) - 0.5).to(torch.bfloat16)
        B = (torch.rand(N, K, device=dev, generator=g) - 0.5).to(torch.bfloat16)
        C = torch.empty(M, N, device=dev, dtype=torch.float32)
        A8, B8 = A.to(torch.float8_e4m3fn), B.to(torch.float8_e4m3fn)
        flops = 2.0 * M * N * K
        res = {"M": M, "N": N, "K": K}
        cases = []
        for c in (1, 2, 3):  # per-tile kernel, ring for 1 or 2 CTAs per SM; 3 = persistent kernel
            cases += [(f"bf16_c{c}", c, lambda: z.gemm_tc(A.data_ptr(), B.data_ptr(), C.data_ptr(), M, N, K, False,
                                                           stream.cuda_stream)),
                      (f"fp8_c{c}", c, lambda: z.gemm_tc(A8.data_ptr(), B8.data_ptr(), C.data_ptr(), M, N, K, True,
                                                          stream.cuda_stream))]
        cases.append(("cublas_bf16", 1, lambda: torch.matmul(A, B.t())))
        for name, ctas, fn in cases:
            z.gemm_configure(ctas)
            for _ in range(args.warmup):
                fn()
            ms = []
            for _ in range(args.steps):
                flush.fill_(1)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                e1.synchronize()
                ms.append(e0.elapsed_time(e1))
            t = statistics.median(ms)
            res[name] = {"ms": round(t, 4), "tflops": round(flops / t / 1e9, 1)}
        for kind in ("bf16", "fp8"):
            best = min((1, 2, 3), key=lambda c: res[f"{kind}_c{c}"]["ms"])
            res[kind] = dict(res[f"{kind}_c{best}"], kernel="persistent" if best == 3 else f"per-tile, {best} CTA/SM")
        z.gemm_configure(0)
        ref = (A.float() @ B.float().t())
        z.gemm_tc(A.data_ptr(), B.data_ptr(), C.data_ptr(), M, N, K, False, stream.cuda_stream)
        res["bf16_max_rel_err"] = float(((C - ref).abs().max() / ref.abs().max()).item())
        rows.append(res)
        print(json.dumps(res), file=sys.stderr, flush=True)
        del A, B, C, A8, B8, ref
    if rank == 0:
        head = rows[0]
        peak = peaks.get("bf16_tflops") or 1900.0
        print(json.dumps({
            "metric": "tensor-core GEMM TFLOP/s (move-ordering network, layer 1)", "value": head["bf16"]["tflops"],
            "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": head["bf16"]["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 (fp32 accumulate)", "data": "synthetic (uniform operands)",
            "config": {"workload": "zeta_gemm_tc on the network's shapes", "l2": "flushed between timed steps"},
            "roofline": {"bound": "tensor", "achieved": head["bf16"]["tflops"], "peak": peak, "unit": "TFLOP/s",
                         "frac": round(head["bf16"]["tflops"] / peak, 4), "traffic": None,
                         "peak_source": "MEASURED_PEAKS.json bf16_tflops (cuBLAS burst)"},
            "shapes": rows,
        }), flush=True)
    z.release()


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    ol, ref = _ref_lib()
    if ref is None:
        print(json.dumps({"impl": "reference", "unavailable": "reference kernels (oracle/_ref) not built here"}))
        return
    # the workload positions, made with the oracle's copy of the generator
    import zeta_gb300 as zmod
    w = dict(zmod.WORKLOADS[WORKLOAD])
    boards, stm, depth = ol.make_positions(w["seed"], 256, min_plies=w["min_plies"], max_plies=w["max_plies"],
                                           min_pieces=w["min_pieces"], min_depth=w["min_depth"],
                                           max_depth=w["max_depth"])
    cores = os.cpu_count() or 1
    k = reference_sample_size(cores)
    d3 = np.full(k, 3, dtype=np.int32)
    for _ in range(args.warmup):
        ol.ref_perft_batch(boards[:cores], stm[:cores], d3[:cores], cores)
    t_total, leaves = 0.0, 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        out = ol.ref_perft_batch(boards[:k], stm[:k], d3, cores)
        t_total += time.perf_counter() - t0
        leaves += int(out.sum())
    value = leaves / t_total
    sample = (f"unmodified zetaperft.cl on {cores} host threads, per step the first {k} workload positions "
              f"at depth 3 ({leaves // args.steps} leaves)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_total / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded random playouts)",
        "config": perft_config(w["n"], world),
        "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": cores, "kind": "reference",
                         "sample": sample},
        "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=0, help="positions per GPU (default: the workload's 4096)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the timed CPU baseline (profiling runs)")
    ap.add_argument("--gemm-shapes", default="", help="gemm: comma-separated indices into GEMM_SHAPES (default all)")
    ap.add_argument("--all-promotions", action="store_true",
                    help="perft promotes to all four pieces (not the reference's rule: no CPU baseline or roofline)")
    ap.add_argument("--no-search", action="store_true",
                    help="default workload: leave out the batched-search and learned-ordering blocks")
    ap.add_argument("--ab-n", type=int, default=0,
                    help="learned-ordering A/B: positions (default: the first 512 in the default line, "
                         "all 1024 with --workload learned_ab)")
    ap.add_argument("--ab-depth", type=int, default=8, help="learned-ordering A/B: iterative-deepening depth")
    ap.add_argument("--ab-pairs", type=int, default=3, help="learned-ordering A/B: interleaved plain/learned pairs")
    ap.add_argument("--ab-model", default="", help="learned-ordering A/B: network parameters (default: the committed)")
    ap.add_argument("--workload", choices=["perft_batch", "search_batch", "learned_ab", "gemm", "engine", "smp"],
                    default="perft_batch")
    ap.add_argument("--depth", type=int, default=0, help="search depth (search_batch; default 7)")
    ap.add_argument("--workers", type=int, default=0, help="ABDADA workers per position (0 = sweep)")
    ap.add_argument("--helpers", type=int, default=0, help="helper cap: max workers per position (0 = none)")
    ap.add_argument("--form", type=int, default=0,
                    help="search_batch launch form with --workers: 0 auto, 1 dense, 2 sparse, 3 warp-cooperative")
    ap.add_argument("--tt1-mb", type=int, default=2048, help="smp: transposition table size")
    ap.add_argument("--smp-workers", default="64,128,192,256,384,512,1024", help="smp: worker counts of the sweep")
    ap.add_argument("--deep-every", type=int, default=0,
                    help="smp: every k-th lazy-SMP helper searches one ply deeper (0 = off, the reference's search)")
    ap.add_argument("--tt2-mb", type=int, default=0,
                    help="smp: ABDADA table size (0 = no TT2: helpers randomise their move order instead)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "search_batch" and args.impl == "ours":
        run_search(args)
    elif args.workload == "learned_ab" and args.impl == "ours":
        run_learned_ab(args)
    elif args.workload == "gemm" and args.impl == "ours":
        run_gemm(args)
    elif args.workload == "engine" and args.impl == "ours":
        run_engine(args)
    elif args.workload == "smp" and args.impl == "ours":
        run_smp(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
