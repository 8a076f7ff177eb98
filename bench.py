#!/usr/bin/env python
"""Headline benchmark: FastNSG graph build of a 1M x 128 dataset on one GB300.

Metric: seconds per build of the FastNSG graph of the 1,000,000 x 128
integer-valued mixture (a seeded stand-in for Sift1M) with the reference's
C2 flags (-K 500 -L 500 -S 12 -R 100 --search_L 80 --nsg_R 50 --search_K 500
--massq_S 10 --loop_i 2 --step 10) and --recall 0.99 as the NN-descent stop
rule; the final KNN-graph recall@K (control recall@MAXL, the reference's
evaluate()) is reported with every line.  One step = one full build (NN-descent,
prune + link, entry point, tree_grow, P2K refinement).

  value  device-resident: rows uploaded once before the timed region; each step
         is kcna_build on the resident rows, timed with CUDA events on the
         library's stream.
  e2e    the same build through the C ABI with host buffers: every step copies
         the rows from pinned host memory, builds, and reads the graph back.

--impl reference times the reference's own CPU build of the same workload on
this machine's host cores: the reference compiled from its sources for this
machine (oracle/build_ref.sh), whole 1M-row buildFastNSG runs through its
public API, as many as fit --ref-budget seconds, each timed by the
reference's own CSV "con time".  The GPU arm's cpu_baseline is one such build.
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

METRIC = "1M×128 graph build s @0.99 KNN recall: learned+BF16 vs plain FP32 (1 GB300)"
UNIT = "s"
FLAGS = dict(K=500, L=500, S=12, R=100, iterations=12, search_L=80, nsg_R=50, search_K=500, massq_S=10,
             loop_i=2, step=10, angle=60.0, recall=0.99, controls=100, seed=2024)


def static_config(n):
    """The workload, identical in the GPU arm and the reference arm."""
    return {"workload": "c2 FastNSG 1M x 128 (integer-valued 256-cluster mixture)", "n": n,
            "l2_policy": "inputs larger than L2 (rows 512 MB, pools 4 GB)", **FLAGS}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), float(j.get("bf16_tflops_sustained", j["bf16_tflops"])), "measured"
    except Exception:
        return 6800.0, 1700.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=ws)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _reference_lib():
    """The reference compiled from its own sources for this machine
    (oracle/build_ref.sh, run by build()), or None with the reason."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    if not oracle_py.Reference.available():
        return None, "oracle/_ref/libkcna_ref.so is absent (the reference sources were not staged here)"
    try:
        return oracle_py.Reference(), None
    except OSError as e:  # built for another architecture
        return None, f"oracle/_ref/libkcna_ref.so does not load here: {e}"


def reference_builds(X, threads, budget_s, max_builds):
    """Whole FastNSG builds of X by the reference (buildFastNSG through its
    public API, src/kgraph.cpp:3796-3851), as many as fit budget_s (at least
    one, at most max_builds).  Each build's time is the reference's own CSV
    "con time" (last entry: from the start of buildFastNSG to the end of the
    last buildNSG, src/kgraph.cpp:3797,3823-3826).  Returns (builds, graph of
    the last build, kind, note); without a loadable reference the oracle port
    builds instead (kind "port", its own wall time)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    ref, why = _reference_lib()
    p = oracle_py.params(**{**FLAGS, "nthreads": threads})
    builds, graph = [], None
    t_all = time.perf_counter()
    while len(builds) < max(1, max_builds):
        t0 = time.perf_counter()
        if ref is not None:
            sys.stdout.flush()
            saved = os.dup(1)  # the reference prints progress with printf
            devnull = os.open(os.devnull, os.O_WRONLY)
            os.dup2(devnull, 1)
            try:
                rows, ep, width, csv = ref.build(oracle_py.KCNA_NSG, X, p, nthreads=threads)
            finally:
                import ctypes

                ctypes.CDLL(None).fflush(None)  # drain C stdio into /dev/null before restoring
                os.dup2(saved, 1)
                os.close(saved)
                os.close(devnull)
            wall = time.perf_counter() - t0
            r = oracle_py.parse_run_csv(csv)
            con = r.get("con time", [])
            builds.append(dict(seconds=con[-1] if con else wall, wall=wall, recall=r.get("recall", []),
                               con_time=con, aod=(r.get("AOD") or [None])[0]))
            graph = (rows, ep, width)
        else:
            O = oracle_py.Oracle()
            gi, deg, st = O.build(oracle_py.KCNA_NSG, X, p, width=2 * FLAGS["nsg_R"] + 64, nthreads=threads)
            wall = time.perf_counter() - t0
            rec = list(st.iter_recall[: st.iterations]) + list(st.loop_recall[1: st.loops])
            builds.append(dict(seconds=wall, wall=wall, recall=rec, con_time=[], aod=int(st.aod)))
            graph = ([gi[i, : deg[i]] for i in range(gi.shape[0])], int(st.ep), int(st.width))
        elapsed = time.perf_counter() - t_all
        if elapsed + builds[-1]["wall"] > budget_s:
            break
    kind = "reference" if ref is not None else "port"
    return builds, graph, kind, why


def exact_knn_host(X, Q, k, chunk=256):
    """Exact k-NN of Q in X on the host (numpy), ties broken by the lower id.
    Squared L2 from |x|^2 + |q|^2 - 2<x, q> in float64."""
    X64 = X.astype(np.float64)
    xn = (X64 * X64).sum(1)
    out = np.empty((Q.shape[0], k), np.int64)
    for s in range(0, Q.shape[0], chunk):
        q = Q[s: s + chunk].astype(np.float64)
        d = xn[None, :] + (q * q).sum(1)[:, None] - 2.0 * (q @ X64.T)
        part = np.argpartition(d, k, axis=1)[:, : k + 1]
        for i in range(q.shape[0]):
            c = part[i]
            o = np.lexsort((c, d[i, c]))[:k]
            out[s + i] = c[o]
    return out


def reference_search_recall10(X, graph, Q, truth, L=100):
    """Search recall@10 of the reference's own graph with the reference's own
    beam search (get_neighbors, src/kgraph.cpp:1560-1623), started from the
    entry point + L-1 seeded random nodes as in the GPU arm's measurement."""
    rows, ep, width = graph
    n = X.shape[0]
    W = max(1, max(len(r) for r in rows))
    g = np.full((n, W), 0xFFFFFFFF, np.uint32)
    deg = np.zeros(n, np.uint32)
    for i, r in enumerate(rows):
        g[i, : len(r)] = r
        deg[i] = len(r)
    rng = np.random.default_rng(7)
    extra = rng.choice(n, size=L, replace=False)
    start = np.concatenate([[ep], extra[extra != ep][: L - 1]]).astype(np.uint32)
    init = np.broadcast_to(start, (Q.shape[0], L)).copy()
    ref, _ = _reference_lib()
    if ref is None:
        return None
    found, _ = ref.beam_search(X, g, deg, Q, init, L, 10)
    hit = sum(len(set(f.tolist()) & set(t.tolist())) for f, t in zip(found, truth))
    return hit / (10.0 * Q.shape[0])


def run_reference(args, ws, rank):
    """The reference's own CPU build of the same workload on this machine's host
    cores: whole builds of the named size, as many as fit --ref-budget seconds."""
    if rank != 0:
        return
    from fastkcna_gb300 import synth

    threads = os.cpu_count() or 1
    X = synth.base("c2", args.n)
    builds, graph, kind, why = reference_builds(X, threads, args.ref_budget, args.steps)
    v = statistics.median(b["seconds"] for b in builds)
    Q = synth.queries("c2", 10000)
    truth = exact_knn_host(X, Q, 10)
    rec10 = reference_search_recall10(X, graph, Q, truth) if kind == "reference" else None
    sample = (f"{len(builds)} whole FastNSG build(s) of the {args.n:,}-row workload (same flags), "
              f"{threads} host threads, seconds from the reference's CSV con time")
    if kind == "port":
        sample = f"oracle port (the reference does not load here: {why}); " + sample.replace(
            "seconds from the reference's CSV con time", "wall seconds")
    last = builds[-1]
    print(json.dumps({
        "metric": METRIC, "value": round(v, 3), "unit": UNIT, "n_gpus": ws, "steps": len(builds),
        "warmup": 0, "ms_per_step": round(v * 1000, 1), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": static_config(args.n),
        "impl": "reference", "mode": f"reference CPU build ({kind})",
        "cpu_baseline": {"value": round(v, 3), "unit": UNIT, "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": round(v, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "results": {"build_seconds": [round(b["seconds"], 3) for b in builds],
                    "build_wall_seconds": [round(b["wall"], 3) for b in builds],
                    "con_time": [round(x, 3) for x in last["con_time"]],
                    "recall_per_iteration_and_loop": [round(x, 5) for x in last["recall"]],
                    "knn_recall_at_K": round(last["recall"][-1], 5) if last["recall"] else None,
                    "avg_degree": last["aod"],
                    "search_recall_at_10": round(rec10, 4) if rec10 is not None else None,
                    "search": "10,000 queries, the reference's own beam search (get_neighbors), beam 100 from the "
                              "entry point + 99 seeded random nodes, exact 10-NN",
                    "host": {"machine": os.uname().machine, "threads": threads},
                    "warmup_note": "no warm-up build: one build takes minutes and its first-touch of memory is "
                                   "part of the reference's own build"},
    }), flush=True)


def roofline(st, hbm_gbs, ld, n, search_k, tensor_tflops=None):
    """Dominant device phase with its algorithmic bytes per launch.

    join:  every gathered row once (BF16 or FP32) + every candidate's key and
           joiner written once (12 bytes)
    merge: candidates read once, pool entries read and written once
    prune: every candidate row of every pruned node read once (min(pool,
           search_K) rows); the prunes after the first re-prune only the nodes
           whose pool prefix changed (loops x n - prune_skipped nodes in all)
    The Gram-tile prune is also held against the tensor roof: its algorithmic
    work is one BF16 dot product of ld terms per unordered candidate pair,
    c (c - 1) / 2 pairs per node with c = min(pool, search_K) (the tiles it
    issues cover the lower triangle of ceil(c / 128)^2 128 x 128 blocks, about
    1.3 times that).  `bound` names the roof with the longer ideal time; both
    are listed under `roofs`.  None of the phases runs at a roof; `limiter`
    names what the ncu captures under profiles/ show binds each.
    """
    ph, launches = st["phase_ms"], st["phase_launches"]
    rb = 2 if st["bf16_rows"] else 4
    c = min(search_k, st["maxl"])
    pruned = max(st.get("loops", 1) * n - st.get("prune_skipped", 0), 0)  # node prunes run
    models = {
        "join": st["join_rows"] * ld * rb + st["cand_emitted"] * 12,
        "merge": st["cand_merged"] * 8 + st["pool_entries_merged"] * 16,
        "prune": pruned * c * ld * rb,
    }
    kernels = {"join": "join_tc_kernel" if st["gram_tc"] else "join_kernel", "merge": "merge_warp_kernel",
               "prune": "prune_gram_kernel" if st.get("prune_tc") else "prune_kernel"}
    limiters = {
        "join": "scattered 16-byte candidate-slot stores and the TMEM re-read of the write pass (latency, LSU)",
        "merge": "shared-memory latency: binary search of every candidate in the node's pool (bank conflicts)",
        "prune": "issue slots of the mask-building warps; tensor pipe about 30 % busy" if st.get("prune_tc")
        else "latency of the sequential occlusion scan",
    }
    name = max(models, key=lambda k: ph.get(k, 0.0))
    ms, nl = ph[name], max(launches[name], 1)
    per_launch_bytes = models[name] / nl
    per_launch_s = ms / 1000.0 / nl
    achieved = per_launch_bytes / per_launch_s / 1e9 if per_launch_s > 0 else 0.0
    hbm = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_gbs, "unit": "GB/s",
           "frac": round(achieved / hbm_gbs, 4), "algorithmic_per_launch": round(per_launch_bytes / 1e9, 3),
           "algorithmic_unit": "GB"}
    roofs = {"hbm": hbm}
    primary = hbm
    if name == "prune" and st.get("prune_tc") == 1 and tensor_tflops:
        flops = pruned * (c * (c - 1) / 2) * 2.0 * ld / nl  # per launch
        t_achieved = flops / per_launch_s / 1e12 if per_launch_s > 0 else 0.0
        roofs["tensor"] = {"bound": "tensor", "achieved": round(t_achieved, 1), "peak": tensor_tflops,
                           "unit": "TFLOP/s", "frac": round(t_achieved / tensor_tflops, 4),
                           "algorithmic_per_launch": round(flops / 1e12, 3), "algorithmic_unit": "TFLOP"}
        if flops / (tensor_tflops * 1e12) > per_launch_bytes / (hbm_gbs * 1e9):
            primary = roofs["tensor"]
    out = {k: primary[k] for k in ("bound", "achieved", "peak", "unit", "frac")}
    out.update({"traffic": None,
                "traffic_note": "DRAM bytes are not measured by this run (ncu captures are separate)",
                "kernel": kernels[name], "phase": name, "launches_per_step": int(nl),
                "limiter": limiters[name], "roofs": roofs})
    return name, out


def cluster_starts(xlab, qlab, ep, L):
    """Start nodes per query: the entry point and L - 1 seeded random rows of
    the mixture component the query was drawn from."""
    order = np.argsort(xlab, kind="stable")
    bounds = np.searchsorted(xlab[order], np.arange(int(xlab.max()) + 2))
    out = np.empty((len(qlab), L), np.uint32)
    out[:, 0] = ep
    for qi, c in enumerate(qlab):
        members = order[bounds[c]:bounds[c + 1]] if c + 1 < len(bounds) else order[:0]
        if len(members) == 0:
            members = order
        out[qi, 1:] = np.random.default_rng(qi).choice(members, size=L - 1, replace=len(members) < L - 1)
    return out


def search_recall10_in_cluster(ix, Q, truth, xlab, qlab, L=16):
    """Search recall@10 with beams started inside each query's own cluster
    (the entry point plus L - 1 seeded rows of the query's mixture
    component).  C2's clusters are islands of the graph at 1M rows, so the
    entry-point search above mostly measures whether a start lands in the
    query's cluster; this one measures the graph."""
    _, _, ep = ix.graph()
    found, _ = ix.search(Q, L, 10, init_ids=cluster_starts(xlab, qlab, ep, L))
    hit = sum(len(set(f.tolist()) & set(t.tolist())) for f, t in zip(found, truth))
    return hit / (10.0 * Q.shape[0])


def search_recall10(ix, Q, truth, n, L=100):
    """Index search recall@10 of the context's graph: beam of L from the entry
    point plus L-1 seeded random nodes (the same start for every query and
    build), against the exact 10-NN; and the queries per second of that batched
    GPU beam search through the C ABI (host query and result buffers, median of
    3 timed calls after one untimed)."""
    _, _, ep = ix.graph()
    rng = np.random.default_rng(7)
    extra = rng.choice(n, size=L, replace=False)
    start = np.concatenate([[ep], extra[extra != ep][: L - 1]]).astype(np.uint32)
    init = np.broadcast_to(start, (Q.shape[0], L)).copy()
    found, _ = ix.search(Q, L, 10, init_ids=init)
    times = []
    for _ in range(3):
        t0 = time.perf_counter()
        ix.search(Q, L, 10, init_ids=init)
        times.append(time.perf_counter() - t0)
    hit = sum(len(set(f.tolist()) & set(t.tolist())) for f, t in zip(found, truth))
    return hit / (10.0 * Q.shape[0]), Q.shape[0] / statistics.median(times)


def run_search_sweep(args, local):
    """Query-time search over the graphs of both builds (learned+BF16 and plain
    FP32) at beam widths 10-320: recall@10 against the exact 10-NN, the same
    with ties at the 10th distance counted as hits, and queries per second.
    One JSON line; not the timed build measurement."""
    from fastkcna_gb300 import kcna, synth

    n = args.n
    X = synth.base("c2", n)
    Q = synth.queries("c2", 10000)
    ix = kcna.Index(local)
    ix.upload(X)
    truth, tdist = ix.knn_queries(Q, 10)
    curves = {}
    for mode in ("learned_bf16", "plain"):
        p = kcna.params(**FLAGS, **(dict(learned_seed=1, screen=1) if mode == "learned_bf16" else {}))
        ix.build("nsg", p)
        _, _, ep = ix.graph()
        rows = []
        for L in (10, 20, 40, 80, 100, 160, 320):
            rng = np.random.default_rng(7)
            extra = rng.choice(n, size=L, replace=False)
            start = np.concatenate([[ep], extra[extra != ep][: L - 1]]).astype(np.uint32)
            init = np.broadcast_to(start, (Q.shape[0], L)).copy()
            found, fd = ix.search(Q, L, 10, init_ids=init)
            times = []
            for _ in range(3):
                t0 = time.perf_counter()
                ix.search(Q, L, 10, init_ids=init)
                times.append(time.perf_counter() - t0)
            rec = sum(len(set(f.tolist()) & set(t.tolist())) for f, t in zip(found, truth)) / (10.0 * Q.shape[0])
            ties = float(np.mean(np.minimum((fd <= tdist[:, 9:10]).sum(1), 10) / 10.0))
            rows.append(dict(L=L, recall10=round(rec, 4), recall10_ties=round(ties, 4),
                             qps=round(Q.shape[0] / statistics.median(times))))
        curves[mode] = rows
    print(json.dumps({"search_sweep": curves, "n": n, "queries": int(Q.shape[0]),
                      "start": "entry point + L-1 seeded random nodes"}), flush=True)


C3_FLAGS = dict(K=200, L=200, S=10, R=100, iterations=6, search_L=40, nsg_R=40, search_K=200, massq_S=10,
                loop_i=2, step=10)
C4_FLAGS = dict(K=500, L=500, S=12, R=100, iterations=6, search_L=80, nsg_R=50, search_K=500, massq_S=10,
                loop_i=2, step=10, tau=10.0)
C5_FLAGS = dict(K=500, L=500, S=12, R=100, iterations=12, search_L=80, nsg_R=50, search_K=500, massq_S=10,
                loop_i=2, step=10, angle=60.0, recall=0.99)


def _recall10(found, truth):
    return sum(len(set(f.tolist()) & set(t.tolist())) for f, t in zip(found, truth)) / (10.0 * truth.shape[0])


def _search_from_entry(ix, Q, truth, n, ep, L, labels=None):
    rng = np.random.default_rng(7)
    extra = rng.choice(n, size=L, replace=False)
    start = np.concatenate([[ep], extra[extra != ep][: L - 1]]).astype(np.uint32)
    found, _ = ix.search(Q, L, 10, init_ids=np.broadcast_to(start, (Q.shape[0], L)).copy())
    if labels is not None:
        found = labels[found]
    return _recall10(found, truth)


def run_workload(args, local):
    """The other named workloads at full size, one JSON line each (not the
    headline measurement): c3 = the layered FastHNSW command line on 1M x 96
    unit rows, FP32 and BF16-screened; c4 = FastTauMNG on 1M x 960, plain FP32
    and with the FP8 E4M3-screened prune; c5 = FastAlphaPG on 2M x 128 integer
    rows, learned+BF16 and plain FP32.  Times are one build each after the data is on the device
    (c3: the command line's own indexing time, file load excluded)."""
    import tempfile

    import torch

    from fastkcna_gb300 import build as kbuild
    from fastkcna_gb300 import index_io, kcna, synth

    torch.cuda.set_device(local)
    w = args.workload
    out = {"workload": w}
    size = None if args.n == 1_000_000 else args.n  # --n scales c3 / c4 / c5 down (profiling cases)
    out["n"] = size or {"c3": 1_000_000, "c4": 1_000_000, "c5": 2_000_000}[w]
    if w == "c3":
        X = synth.base("c3", size)
        Q = synth.queries("c3", 10000)
        with kcna.Index(local) as ix:
            ix.upload(X)
            truth, _ = ix.knn_queries(Q, 10)
        td = tempfile.mkdtemp()
        data = os.path.join(td, "c3.lshkit")
        synth.write_lshkit(data, X)
        flags = []
        for k, v in C3_FLAGS.items():
            flags += [f"--{k}" if len(k) > 1 else f"-{k}", str(v)]
        flags = [f.replace("--iterations", "-I") for f in flags]
        for screen in ("fp32", "bf16"):
            path = os.path.join(td, f"c3_{screen}.bin")
            t0 = time.perf_counter()
            r = subprocess.run([os.path.join(kbuild.BIN, "fasthnsw"), data, path, "--result",
                                os.path.join(td, f"c3_{screen}.csv"), "--screen", screen, *flags],
                               capture_output=True, text=True, timeout=3000)
            wall = time.perf_counter() - t0
            if r.returncode != 0:
                raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])
            secs = [float(ln.split(":")[-1]) for ln in r.stdout.splitlines() if "indexing time" in ln]
            idx = index_io.read_hnswlib(path)
            labels = np.asarray(idx["labels"], np.uint32)
            W = max(len(a) for a in idx["level0"])
            g = np.full((X.shape[0], W), 0xFFFFFFFF, np.uint32)
            deg = np.zeros(X.shape[0], np.uint32)
            for i, a in enumerate(idx["level0"]):
                g[i, : len(a)] = a
                deg[i] = len(a)
            with kcna.Index(local) as ix:
                ix.upload(X[labels])
                ep = int(idx["enterpoint"])
                ix.set_graph(g, deg, ep)
                rec = {L: round(_search_from_entry(ix, Q, truth, X.shape[0], ep, L, labels), 4) for L in (40, 100)}
            out[screen] = {"indexing_s": secs[-1] if secs else None, "wall_s": round(wall, 2),
                           "level0_avg_degree": round(float(deg.mean()), 2), "search_recall_at_10": rec}
        out["flags"] = C3_FLAGS
        out["search"] = "level-0 graph, beam L from the entry point + L-1 seeded random nodes, 10,000 queries"
    elif w == "c4":
        X = synth.base("c4", size)
        Q = synth.queries("c4", 1000)
        with kcna.Index(local) as ix:
            ix.upload(X)
            truth, _ = ix.knn_queries(Q, 10)
            # plain FP32, then the FP8 E4M3-screened prune (BF16 mode at d >= 256)
            for mode, extra in (("fp32", {}), ("fp8_screen", dict(screen=1))):
                t0 = time.perf_counter()
                st = ix.build("taumng", kcna.params(**C4_FLAGS, **extra))
                wall = time.perf_counter() - t0
                _, deg, ep = ix.graph()
                rec = {L: round(_search_from_entry(ix, Q, truth, X.shape[0], ep, L), 4) for L in (80, 160)}
                out[mode] = dict(build_s=round(st["total_time"], 3), wall_s=round(wall, 3),
                                 phase_ms={k: round(v, 1) for k, v in st["phase_ms"].items() if v},
                                 nndescent_iterations=st["iterations"],
                                 knn_recall_at_K=round(st["loop_recall"][-1], 4), n_comps=st["n_comps"],
                                 cand_emitted=st["cand_emitted"], prune_comps=st["prune_comps"],
                                 bridge_comps=st["bridge_comps"], prune_tc=st["prune_tc"],
                                 prune_exact_pairs=st["prune_exact"], avg_degree=st["aod"],
                                 search_recall_at_10=rec)
        out["ratio"] = round(out["fp8_screen"]["build_s"] / out["fp32"]["build_s"], 4)
        out["flags"] = C4_FLAGS
    elif w == "c5":
        X = synth.base("c5", size)
        with kcna.Index(local) as ix:
            ix.upload(X)
            for mode, extra in (("learned_bf16", dict(learned_seed=1, screen=1)), ("plain", {})):
                st = ix.build("alphapg", kcna.params(**C5_FLAGS, **extra))
                out[mode] = dict(build_s=round(st["total_time"], 3), iterations=st["iterations"],
                                 iter_recall=[round(x, 4) for x in st["iter_recall"]],
                                 knn_recall_at_K=round(st["loop_recall"][-1], 4),
                                 phase_ms={k: round(v, 1) for k, v in st["phase_ms"].items() if v})
        out["ratio"] = round(out["learned_bf16"]["build_s"] / out["plain"]["build_s"], 4)
        out["flags"] = C5_FLAGS
    print(json.dumps(out), flush=True)


def run_gpu(args, ws, rank, local):
    import torch

    from fastkcna_gb300 import kcna, synth

    torch.cuda.set_device(local)
    n = args.n
    X, xlab = synth.base_labels("c2", n)
    mode = dict(learned_seed=1, screen=1) if args.mode == "learned_bf16" else {}
    p = kcna.params(**FLAGS, **mode)
    p_plain = kcna.params(**FLAGS)
    ix = kcna.Index(local)
    stream = torch.cuda.ExternalStream(ix.stream, device=torch.device("cuda", local))
    ix.upload(X)
    for _ in range(args.warmup):
        ix.build("nsg", p)
    # the plain FP32 build, timed the same way, for the learned+BF16 vs plain comparison
    plain_ms = None
    if args.mode == "learned_bf16":
        ix.build("nsg", p_plain)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plain_stats = [ix.build("nsg", p_plain) for _ in range(args.steps)]
        e1.record(stream)
        e1.synchronize()
        plain_ms = e0.elapsed_time(e1) / args.steps
        Q, qlab = synth.query_labels("c2", 10000)
        truth, _ = ix.knn_queries(Q, 10)
        plain_rec10, plain_qps = search_recall10(ix, Q, truth, n)
        plain_rec10_c = search_recall10_in_cluster(ix, Q, truth, xlab, qlab)
        ix.build("nsg", p)
    # timed region: device-resident rows, one build per step
    clock = ClockSampler(local)
    clock.start()
    barrier(ws)
    torch.cuda.synchronize()
    launches0 = ix.launches
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    stats = []
    for _ in range(args.steps):
        stats.append(ix.build("nsg", p))
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    barrier(ws)
    clocks = clock.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    launches = (ix.launches - launches0) // args.steps
    ms = max_over_ranks(ws, ms)
    # end-to-end through the C ABI with host buffers (pinned)
    Xh = torch.empty((n, X.shape[1]), dtype=torch.float32, pin_memory=True)
    Xh.numpy()[:] = X
    W = None
    e2e = []
    for i in range(args.steps + 1):
        barrier(ws)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rc = ix.lib.kcna_upload(ix.h, Xh.data_ptr(), n, X.shape[1], X.shape[1] * 4)
        if rc != 0:
            raise RuntimeError(f"kcna_upload failed: {rc}")
        ix.build("nsg", p)
        g, deg, ep = ix.graph()
        e1.record(stream)
        e1.synchronize()
        if i > 0:  # first e2e step re-warms the allocator
            e2e.append(e0.elapsed_time(e1) / 1000.0)
        W = g.shape[1]
    e2e_s = max_over_ranks(ws, statistics.median(e2e))
    st = stats[-1]
    if plain_ms is None:
        Q, qlab = synth.query_labels("c2", 10000)
        truth, _ = ix.knn_queries(Q, 10)
        plain_rec10 = plain_rec10_c = None
    rec10, qps = search_recall10(ix, Q, truth, n)  # the graph of the last (end-to-end) build
    rec10_c = search_recall10_in_cluster(ix, Q, truth, xlab, qlab)
    hbm, bf16, src = peaks()
    kname, roof = roofline(st, hbm, (X.shape[1] + 3) // 4 * 4, n, FLAGS["search_K"], tensor_tflops=bf16)
    roof["peak_source"] = (f"{src} (MEASURED_PEAKS.json hbm_gbs; bf16_tflops_sustained for the tensor roof: "
                           "the kernel is timed inside a build of about a second)" if src == "measured"
                           else "fallback 6.8 TB/s, 1.7 PFLOP/s sustained bf16")
    final_recall = st["loop_recall"][-1]
    line = {
        "metric": METRIC, "value": round(ms / 1000.0, 4), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 2), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": static_config(n),
        "mode": "learned seed + BF16" if args.mode == "learned_bf16" else "plain FP32",
        "parallelism": "replicas" if ws > 1 else "single GPU",
        "results": {"knn_recall_at_K": round(final_recall, 4),
                    "nndescent_iterations": st["iterations"],
                    "nndescent_recall": [round(x, 4) for x in st["iter_recall"]],
                    "loop_recall": [round(x, 4) for x in st["loop_recall"]],
                    "phase_ms": {k: round(v, 2) for k, v in st["phase_ms"].items() if v},
                    "dist_evals_per_s": round((st["n_comps"] + st["prune_comps"] + st["bridge_comps"]) / (ms / 1000.0)),
                    "cand_overflow": sum(st["iter_cand_overflow"]), "cand_emitted": st["cand_emitted"],
                    "cand_merged": st["cand_merged"], "tree_attached": st["tree_attached"],
                    "prune_skipped": st["prune_skipped"],
                    "avg_degree": st["aod"],
                    "iter_join_ms": [round(x, 1) for x in st["iter_join_ms"]],
                    "iter_merge_ms": [round(x, 1) for x in st["iter_merge_ms"]],
                    "iter_cand_M": [round(x / 1e6, 1) for x in st["iter_cand"]],
                    "iter_inserted_M": [round(x / 1e6, 1) for x in st["iter_inserted"]],
                    "iter_cand_overflow_M": [round(x / 1e6, 1) for x in st["iter_cand_overflow"]],
                    "bf16_rows": st["bf16_rows"], "seed_ms": round(st["seed_total_ms"], 1),
                    "seed_train_ms": round(st["seed_train_ms"], 1),
                    "seed_recall": round(st["seed_recall"], 4),
                    "plain_fp32_s": round(plain_ms / 1000.0, 4) if plain_ms else None,
                    "plain_fp32_knn_recall_at_K": round(plain_stats[-1]["loop_recall"][-1], 4) if plain_ms else None,
                    "plain_fp32_nndescent_iterations": plain_stats[-1]["iterations"] if plain_ms else None,
                    "plain_fp32_nndescent_recall": [round(x, 4) for x in plain_stats[-1]["iter_recall"]] if plain_ms else None,
                    "plain_fp32_phase_ms": {k: round(v, 2) for k, v in plain_stats[-1]["phase_ms"].items() if v}
                    if plain_ms else None,
                    "learned_bf16_over_plain": round(ms / plain_ms, 4) if plain_ms else None,
                    "search_recall_at_10": round(rec10, 4),
                    "plain_fp32_search_recall_at_10": round(plain_rec10, 4) if plain_rec10 is not None else None,
                    "search_recall_at_10_in_cluster": round(rec10_c, 4),
                    "plain_fp32_search_recall_at_10_in_cluster":
                        round(plain_rec10_c, 4) if plain_rec10_c is not None else None,
                    "search_qps": round(qps),
                    "plain_fp32_search_qps": round(plain_qps) if plain_ms else None,
                    "search": "10,000 queries, beam 100 from the entry point + 99 seeded random nodes, exact 10-NN; "
                              "in_cluster: beam 16 from the entry point + 15 seeded rows of the query's cluster"},
        "gpu_launches": int(launches),
        "e2e": {"value": round(e2e_s, 4), "unit": UNIT, "h2d_bytes_per_step": int(n * X.shape[1] * 4),
                "d2h_bytes_per_step": int(n * W * 4 + n * 4 + 8)},
        "roofline": roof,
        "clocks": clocks,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        builds, _, kind, why = reference_builds(X, threads, 0.0, 1)
        b = builds[0]
        line["cpu_baseline"] = {
            "value": round(b["seconds"], 3), "unit": UNIT, "cores": threads, "kind": kind,
            "sample": ("one whole FastNSG build of the same 1M-row workload and flags by the reference compiled "
                       "from its sources for this host, seconds from its CSV con time" if kind == "reference" else
                       f"one whole FastNSG build of the same 1M-row workload by the oracle port ({why}), wall seconds"),
            "knn_recall_at_K": round(b["recall"][-1], 5) if b["recall"] else None}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ix.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--ref-budget", type=float, default=600.0,
                    help="seconds of whole reference builds in --impl reference (at least one build)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="learned_bf16", choices=["learned_bf16", "plain"])
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c4", "c5"],
                    help="c2: the headline build benchmark; c3/c4/c5: one JSON line for that named workload")
    ap.add_argument("--search-sweep", action="store_true",
                    help="print the recall@10 / QPS curve of the query-time search instead of timing builds")
    args = ap.parse_args()
    ws, rank, local = dist_setup()
    if args.workload != "c2":
        if rank == 0:
            run_workload(args, local)
    elif args.search_sweep:
        if rank == 0:
            run_search_sweep(args, local)
    elif args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_gpu(args, ws, rank, local)


if __name__ == "__main__":
    main()
