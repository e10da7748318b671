#!/usr/bin/env python
"""SCC GTEPS on R-MAT-24 on one GB300, beside the reference's OpenMP Multistep.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbconn|reference]

A step is one full SCC run (trim, FW-BW, colour rounds, canonical labels) of
the directed R-MAT graph of scale 24, edge factor 16 (a=0.57 b=0.19 c=0.19,
seed 1, self-loops and duplicates removed: 16,777,216 vertices,
263,434,267 edges), the workload the headline metric is quoted on.  GTEPS =
edges / seconds per step.

value : the CSR and its pull hints already resident in HBM, labels written
        to device memory, steps enqueued back to back, CUDA events on the
        library's stream.  value_no_hints: the same steps on the graph with
        its hints freed (what gb_run_scc, which builds no hints, runs).
e2e   : the reference-shaped C-ABI call gb_run_scc (the run_scc signature
        with the reference's 32-bit CSR layout) on pinned host buffers: every
        step reads the out-CSR, both offset arrays and the in-lists of the
        last fifth of the in-edges from host memory (the others are derived
        on the device from the out-CSR) and writes the labels
        device->host; e2e.by_share: the same with the in-lists all copied
        (0.0) or all derived (1.0).
wcc   : WCC (run_cc on the mirrored graph) of the same graph: gb_wcc device
        resident, and gb_run_cc end to end on the mirrored 32-bit CSR (read
        in place by a sampled union-find that skips most of the largest
        component's lists).
Parity: the canonical labels' SHA-256 and the verify lines are compared with
the reference's own (tests/golden/pins.json, made by running the unmodified
reference on the same edge list).
For N > 1 (torchrun) every rank runs a replica on its own GPU ("replicas
only": the path does not shard), barrier + max time over ranks.

grid   : the 4096^2 oriented lattice with chains (config 3), labels checked
         against the reference's digests.
batched: 20,000 R-MAT graphs (vertex counts log-normal, median 2,000, sigma
        1.5, clipped to 64..500,000; edge factor uniform in 4..32) resident
        as one batch; graphs/s of one batched SCC run against back-to-back
        per-graph runs and against the reference (a loop of run_scc).
served: Poisson streams (80% SCC / 20% WCC) at swept rates through
        gb_server from pinned host buffers; p50/p99 latency and graphs/s,
        against the same arrivals served one request at a time by the GPU
        and by the reference.

--impl reference times the reference's own run_scc (the unmodified
multistep/ code, oracle/_ref, built on this host) on all host cores on the
same graph, generated without the product library; each step one run.  Where
the reference is not built it falls back to the C restatement in oracle/.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SCC GTEPS on R-MAT-24 (1 GB300) vs host OpenMP; batched graphs/s and p99 ms"
SCALE, EF, SEED = 24, 16, 1
BATCH_COUNT = 20000
E2E_SHARE = 0.8  # gb_run_scc's default share of in-lists derived on the device
BATCH_DIST = dict(seed=4, median=2000.0, sigma=1.5, n_min=64, n_max=500000, ef_min=4, ef_max=32)
ABC = (0.57, 0.19, 0.19)
PINS = os.path.join(ROOT, "tests", "golden", "pins.json")


def workload_name(n, m, scale=SCALE):
    return (f"R-MAT scale {scale}, edge factor {EF}, a=0.57 b=0.19 c=0.19, seed {SEED}, "
            f"self-loops and duplicates removed ({n:,} vertices, {m:,} edges); SCC")


def config_for(n, m, scale=SCALE, ws=1):
    """The config both arms report (same keys and values)."""
    return {"workload": workload_name(n, m, scale),
            "l2": "inputs larger than L2 (2.1 GB CSR, 129 MB L2); no flush",
            "parallelism": "replicas only" if ws > 1 else "single GPU",
            "trim_level": 1, "labels": "canonical minimum member id",
            "hints": "value: pull hints prebuilt with the graph (k_hint, out and in); "
                     "value_no_hints and e2e: none"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=300)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="gbconn", choices=["gbconn", "reference"])
    p.add_argument("--e2e-steps", type=int, default=20)
    p.add_argument("--cpu-reps", type=int, default=3)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--scale", type=int, default=SCALE,
                   help="R-MAT scale of the headline graph (smaller only for profiling)")
    p.add_argument("--sections", default="headline,grid,batched,served",
                   help="comma list of headline, grid, batched, served")
    p.add_argument("--grid-side", type=int, default=4096,
                   help="lattice side of the grid section (smaller only for profiling)")
    p.add_argument("--serve-rates", default="100,1000,5000,20000,max",
                   help="arrival rates (graphs/s) of the served sweep; max = all at once")
    p.add_argument("--serve-seconds", type=float, default=1.5)
    p.add_argument("--serve-pool", type=int, default=400)
    p.add_argument("--batch-cpu-sample", type=int, default=1000,
                   help="graphs of the batch the reference runs for its CPU figure")
    return p.parse_args()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def pins():
    try:
        with open(PINS) as f:
            return json.load(f)
    except Exception:
        return {}


def edge_digest(n, s, d) -> str:
    import numpy as np
    h = hashlib.sha256()
    h.update(np.int64(n).tobytes())
    h.update(np.ascontiguousarray(s, np.int32).tobytes())
    h.update(np.ascontiguousarray(d, np.int32).tobytes())
    return h.hexdigest()


def label_digest(canonical_labels) -> str:
    import numpy as np
    return hashlib.sha256(np.ascontiguousarray(canonical_labels, "<i4").tobytes()).hexdigest()


def profile_traffic(kernel="k_run"):
    """DRAM bytes per launch of a kernel from the committed ncu summary
    (profiles/traffic.json, R-MAT scale 24), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            d = json.load(f)
        return d.get(f"{kernel}_bytes_per_launch")
    except Exception:
        return None


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the
    timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.index)],
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
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_barrier():
    """Barrier over the ranks of an initialised process group (no-op alone)."""
    import torch.distributed as tdist
    if tdist.is_available() and tdist.is_initialized() and tdist.get_world_size() > 1:
        tdist.barrier()


def dist_max(x: float) -> float:
    """Maximum of x over the ranks (the slowest rank's time); x alone."""
    import torch
    import torch.distributed as tdist
    if not (tdist.is_available() and tdist.is_initialized()) or tdist.get_world_size() == 1:
        return x
    dev = (torch.device("cuda", torch.cuda.current_device()) if tdist.get_backend() == "nccl"
           else torch.device("cpu"))
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def job_gteps(edges_per_rank: int, ranks: int, seconds_max: float, steps: int) -> float:
    """Whole-job GTEPS: every rank runs its own replica, so the job
    processes ranks x edges per step in the slowest rank's time."""
    return ranks * edges_per_rank / (seconds_max / steps) / 1e9


def host_threads() -> int:
    try:
        return int(os.environ.get("OMP_NUM_THREADS", "")) or os.cpu_count()
    except ValueError:
        return os.cpu_count()


# ---------------------------------------------------------------------------
# CPU legs (the reference where it is built on this host, else the port)
# ---------------------------------------------------------------------------
def cpu_scc_baseline(n, s, d, reps):
    """The reference's run_scc on all host cores: best of reps after one
    warm-up, plus one single-thread run.  Returns (canonical labels, verify
    line, best s, cores, one-thread s, kind, what)."""
    import oracle
    cores = host_threads()
    if oracle.ref_available():
        raw, line, times = oracle.ref_run_times("scc", n, s, d, reps=reps + 1)
        _, _, one = oracle.ref_run_times("scc", n, s, d, reps=1, threads=1)
        return (oracle.canonical(raw), line, min(times[1:]), cores, one[0], "reference",
                "the unmodified reference run_scc (multistep/, oracle/_ref), OpenMP")
    cg = oracle.CpuGraph(n, s, d)
    lab = oracle.scc(cg)
    best = 1e30
    for _ in range(reps):
        t0 = time.perf_counter()
        oracle.scc(cg, canonical=False)
        best = min(best, time.perf_counter() - t0)
    oracle.set_threads(1)
    t0 = time.perf_counter()
    oracle.scc(cg, canonical=False)
    one = time.perf_counter() - t0
    oracle.set_threads(cores)
    import connectivity_gb300 as gb
    return (lab, gb.scc_verify(lab), best, cores, one, "port",
            "oracle/multistep.c, OpenMP restatement of run_scc (reference not built here)")


def cpu_cc_baseline(n, s, d, reps):
    """The reference's run_cc on the mirrored graph, all host cores."""
    import oracle
    if oracle.ref_available():
        raw, line, times = oracle.ref_run_times("cc", n, s, d, reps=reps + 1)
        return oracle.canonical(raw), line, min(times[1:]), "reference"
    cg = oracle.CpuGraph(n, s, d, mirror=True)
    lab = oracle.cc(cg)
    best = 1e30
    for _ in range(reps):
        t0 = time.perf_counter()
        oracle.cc(cg, canonical=False)
        best = min(best, time.perf_counter() - t0)
    import connectivity_gb300 as gb
    return lab, gb.cc_verify(lab), best, "port"


def run_reference(args):
    """--impl reference: the reference's run_scc on this host's cores, on the
    same graph (generated by oracle/gen.c, without the product library)."""
    ws, rank, _ = dist()
    if rank != 0:
        return
    import numpy as np

    import oracle
    t0 = time.time()
    n, s, d = oracle.rmat_edges(args.scale, EF, SEED, ABC)
    m = int(s.size)
    prep = time.time() - t0
    pin = pins().get(f"rmat_s{args.scale}_ef{EF}_seed{SEED}", {})
    edges_ok = edge_digest(n, s, d) == pin.get("edges") if pin else None
    W, K = max(args.warmup, 0), max(args.steps, 1)
    cores = host_threads()
    if oracle.ref_available():
        raw, vline, times = oracle.ref_run_times("scc", n, s, d, reps=W + K)
        lab = oracle.canonical(raw)
        kind = "reference"
        what = ("each step one run_scc of the unmodified reference (multistep/, built on this "
                "host by oracle/build_ref.sh) on the workload, OpenMP over all host threads; "
                "the CSR is built once before the steps, as create_csr is outside the "
                "reference's timer")
        T = float(sum(times[W:]))
    else:
        cg = oracle.CpuGraph(n, s, d)
        for _ in range(W):
            oracle.scc(cg, canonical=False)
        t1 = time.perf_counter()
        for _ in range(K):
            oracle.scc(cg, canonical=False)
        T = time.perf_counter() - t1
        lab = oracle.scc(cg)
        vline = None
        kind = "port"
        what = ("each step one run of oracle/multistep.c (OpenMP restatement of run_scc; the "
                "reference is not built on this host)")
    val = m / (T / K) / 1e9
    parity = {"edges_digest_equal_reference_pin": edges_ok}
    if pin:
        parity["scc_digest_equal_reference_pin"] = label_digest(lab) == pin.get("scc_labels")
        if vline is not None:
            parity["verify_line"] = vline.strip()
    line = {
        "impl": "reference", "metric": METRIC, "value": round(val, 4), "unit": "GTEPS",
        "n_gpus": args.gpus, "steps": K, "warmup": W,
        "ms_per_step": round(T / K * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": config_for(n, m, args.scale, ws),
        "graph_build_s": round(prep, 1),
        "cpu_baseline": {"value": round(val, 4), "unit": "GTEPS", "cores": cores, "kind": kind,
                         "sample": what,
                         "host": {"nproc": os.cpu_count(), "machine": os.uname().machine}},
        "e2e": {"value": round(val, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "parity": parity,
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# sections of the GPU arm
# ---------------------------------------------------------------------------
def batched_section(gb, ctx, stream, steps, cpu_sample, want_cpu, ws=1, rank=0):
    """graphs/s of one batched SCC run over BATCH_COUNT resident graphs,
    against back-to-back per-graph runs of a sample of the same graphs, and
    against the reference's loop of run_scc over a sample.  Under torchrun
    the batch is sharded over the ranks (one GPU each, no collective): every
    rank runs the union of its own graphs, and the job's graphs/s is the
    whole batch over the slowest rank's time."""
    import numpy as np
    import torch
    ns, efs, seeds = gb.batch_sizes(BATCH_COUNT, **BATCH_DIST)
    shard_info = None
    if ws > 1:
        from connectivity_gb300 import shard
        of, load = shard.plan(shard.graph_costs(ns, ns.astype(np.int64) * efs), ws)
        idx = shard.members(of, rank)
        ns, efs, seeds = ns[idx], efs[idx], seeds[idx]
        shard_info = {"shards": ws, "plan": "gb_shard_plan on vertices + edge-factor x vertices",
                      "max_over_mean_load": round(float(load.max() / load.mean()), 4)}
    t0 = time.time()
    b = gb.Batch.rmat(ctx, ns, efs, seeds)
    build_s = time.time() - t0
    labels = torch.empty(max(b.n, 1), dtype=torch.int32, device="cuda")
    o = gb.opts()
    for _ in range(3):
        ctx.batch_scc_async(b, labels.data_ptr(), o)
    ctx.sync()
    K = max(1, steps)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(K):
        ctx.batch_scc_async(b, labels.data_ptr(), o)
    e1.record(stream)
    torch.cuda.synchronize()
    ctx.sync()
    t_scc = dist_max(e0.elapsed_time(e1) / 1e3 / K)
    batch_lab = labels[:b.n].cpu().numpy()
    wl = torch.empty_like(labels)
    ctx.batch_wcc(b, labels=wl.data_ptr())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(K):
        ctx.batch_wcc(b, labels=wl.data_ptr())
    t_wcc = (time.perf_counter() - t0) / K
    # per-graph launches: every graph in turn (the first `S`), resident, with
    # the committed size-class options (each graph's own class)
    from connectivity_gb300 import tune as gbtune
    gbtune.install(ctx)
    S = min(2000, b.count)
    gs = [gb.Graph.rmat_n(ctx, int(ns[i]), int(efs[i]), int(seeds[i])) for i in range(S)]
    outs = [torch.empty(max(g.n, 1), dtype=torch.int32, device="cuda") for g in gs]
    for g, lab in zip(gs[:20], outs[:20]):
        ctx.scc_async(g, lab.data_ptr())
    ctx.sync()
    e0.record(stream)
    for g, lab in zip(gs, outs):
        ctx.scc_async(g, lab.data_ptr())
    e1.record(stream)
    torch.cuda.synchronize()
    ctx.sync()
    t_alone = e0.elapsed_time(e1) / 1e3
    ctx.set_class_opts([], [])
    same = all(np.array_equal(outs[i][:gs[i].n].cpu().numpy(),
                              batch_lab[b.vbase[i]:b.vbase[i + 1]]) for i in range(S))
    for g in gs:
        g.close()
    del outs
    # the autotuner on this batch (device-timed coordinate search)
    from connectivity_gb300 import tune as gbtune
    tuned = gbtune.tune_batch(ctx, b, 0, reps=2)
    out = {
        "workload": (f"{BATCH_COUNT:,} R-MAT graphs, vertex counts log-normal (median 2,000, "
                     f"sigma 1.5, clipped 64..500,000), edge factor uniform 4..32 ({b.n:,} "
                     f"vertices, {b.m:,} edges on this rank), one disjoint-union CSR resident "
                     "in HBM"),
        "graphs_per_s": round(BATCH_COUNT / t_scc, 1), "ms_per_batch": round(t_scc * 1e3, 3),
        "sharded": shard_info,
        "steps": K, "gteps": round(b.m / t_scc / 1e9, 2),
        "wcc_graphs_per_s": round(b.count / t_wcc, 1),
        "per_graph_graphs_per_s": round(S / t_alone, 1),
        "per_graph_sample": (f"first {S} graphs of the batch, resident, gb_scc_async back to back "
                             "with each graph's size-class options (the committed table)"),
        "speedup_vs_per_graph": round((BATCH_COUNT / t_scc) / (S / t_alone) / ws, 1),
        "labels_equal_per_graph_runs": bool(same), "build_s": round(build_s, 2),
        "autotuned": {"graphs_per_s": round(b.count / (tuned["ms"] / 1e3), 1),
                      "defaults_graphs_per_s": round(b.count / (tuned["default_ms"] / 1e3), 1),
                      "opts": tuned["opts"]},
        # the graphs of each vertex-count class as a batch of their own,
        # tuned against the defaults: the most that options chosen per size
        # class could gain inside one merged run
        "per_class_tuning": gbtune.tune_batch_by_class(ctx, ns, efs, seeds, 0, reps=2),
    }
    if want_cpu and cpu_sample > 0:
        import oracle
        C = min(cpu_sample, b.count)
        graphs = [gb.rmat_edges_n(int(ns[i]), int(efs[i]), int(seeds[i])) for i in range(C)]
        edges = int(sum(g[1].size for g in graphs))
        res = {}
        if oracle.ref_available():
            for mode in ("seq", "par"):
                labs, T, _ = oracle.ref_batch("scc", graphs, mode)
                ok = all(np.array_equal(oracle.canonical(labs[i]),
                                        batch_lab[b.vbase[i]:b.vbase[i + 1]]) for i in range(C))
                res[mode] = (C / T, ok)
            kind = "reference"
        else:
            # the port per graph, all threads (its runs are serial in Python)
            t0 = time.perf_counter()
            for (n, s, d) in graphs:
                oracle.scc(oracle.CpuGraph(n, s, d), canonical=False)
            res["seq"] = (C / (time.perf_counter() - t0), None)
            kind = "port"
        gps = res["seq"][0]
        out["cpu_baseline"] = {
            "value": round(gps, 1), "unit": "graphs/s", "cores": host_threads(), "kind": kind,
            "sample": (f"the first {C} graphs of the batch ({edges:,} edges): a loop of run_scc, "
                       "one graph after another, each with all host threads (the reference's "
                       "equivalent of a batch); CSRs built before the timed loop"),
            "labels_equal_batch": res["seq"][1],
        }
        if "par" in res:
            out["cpu_baseline"]["one_thread_per_graph"] = {
                "value": round(res["par"][0], 1), "unit": "graphs/s",
                "labels_equal_batch": res["par"][1],
                "how": "the same graphs spread over all host threads, one thread per graph"}
        out["speedup_vs_cpu_baseline"] = round((b.count / t_scc) / gps, 1)
    b.close()
    return out


def grid_section(gb, ctx, side=4096, reps=2):
    """Config 3: the oriented side x side lattice with chains, where the
    colour rounds do the work.  Device time per run (best of reps after one
    warm-up), the labels against the reference's digests, and the colour
    phase's bytes touched per second against the HBM peak (that phase is
    bound by chains of dependent hops, not by bandwidth)."""
    import torch
    n, s, d = gb.grid_edges(side)
    pin = pins().get(f"grid_{side}_seed2", {})
    g = gb.Graph.from_edges(ctx, n, s, d)
    peak, kind = peaks()
    # (an NVTX range, so that a profiler can select these runs: ncu --nvtx
    # --nvtx-include "grid/")
    torch.cuda.nvtx.range_push("grid")
    out = {"workload": (f"{side}x{side} oriented lattice plus chains, seed 2 ({n:,} vertices, "
                        f"{s.size:,} edges); not part of the headline"),
           "edges_digest_equal_reference_pin": (edge_digest(n, s, d) == pin.get("edges")
                                                if pin else None)}
    for name, fn, pk in (("scc", ctx.scc, "scc"), ("wcc", ctx.wcc, "cc")):
        lab = fn(g)
        runs = [fn(g, stats=True)[1] for _ in range(reps)]
        st = min(runs, key=lambda x: x.ms_total)
        e = {"ms_per_run": round(st.ms_total, 3),
             "phases_ms": {"trim": round(st.ms_trim, 3), "reach": round(st.ms_reach, 3),
                           "colour": round(st.ms_colour, 3)},
             "colour_rounds": int(st.colour_rounds),
             "steps": {"search": int(st.fw_steps + st.bw_steps), "colour": int(st.colour_steps),
                       "mark": int(st.mark_steps)}}
        if pin:
            vline = gb.scc_verify(lab) if name == "scc" else gb.cc_verify(lab)
            e["digest_equal_reference_pin"] = label_digest(lab) == pin.get(f"{pk}_labels")
            e["verify_equal_reference_pin"] = vline == pin.get(f"{pk}_verify")
            e["verify_line"] = vline.strip()
            e["reference_seconds_on_pin_host"] = pin.get(f"{pk}_ref_seconds")
            e["pin_host"] = pin.get("host")
        if st.ms_colour > 0:
            gbs = st.bytes_colour / (st.ms_colour * 1e-3) / 1e9
            e["colour_roofline"] = {"bytes_touched": int(st.bytes_colour),
                                    "achieved_gbs": round(gbs, 1), "peak": peak,
                                    "peak_source": f"{kind} hbm_gbs", "frac": round(gbs / peak, 4),
                                    "bound": "latency (chains of dependent hops)"}
        out[name] = e
    torch.cuda.nvtx.range_pop()
    g.close()
    return out


def _fifo(arr_s, svc):
    """Latencies (s) of arrivals served one at a time, first come first
    served, with the given service times."""
    import numpy as np
    fin = 0.0
    lat = np.zeros(len(arr_s))
    for j in range(len(arr_s)):
        fin = max(arr_s[j], fin) + svc[j]
        lat[j] = fin - arr_s[j]
    return lat, fin


def served_section(gb, device, rates, seconds, pool_size, want_cpu):
    """gb_server under Poisson streams at each rate ("max": every request
    arrives at once, the server's capacity); the same arrivals served one
    launch per request (FIFO over measured per-request GPU service times),
    and by the reference one run_scc / run_cc per request (FIFO over its
    measured per-graph times)."""
    import numpy as np
    import torch
    ns, efs, seeds = gb.batch_sizes(pool_size, **BATCH_DIST)
    pool = []
    for i in range(pool_size):
        n, s, d = gb.rmat_edges_n(int(ns[i]), int(efs[i]), int(seeds[i]))
        pool.append((n, torch.from_numpy(s).pin_memory().numpy(),
                     torch.from_numpy(d).pin_memory().numpy()))
    ctx = gb.Context(device)

    def alone(i, kind, out=None):
        # one request on its own: the one-call path from its edges (one block
        # for a small graph, else a device graph built, run and freed)
        n, s, d = pool[i]
        return ctx.scc_edges(n, s, d, labels=out) if kind == 0 else ctx.wcc_edges(n, s, d,
                                                                                 labels=out)

    for i in range(min(20, pool_size)):
        alone(i, 0)
    svc = np.zeros((pool_size, 2))
    for i in range(pool_size):
        for k in (0, 1):
            t0 = time.perf_counter()
            alone(i, k)
            svc[i, k] = time.perf_counter() - t0
    ref_svc, ref_kind = None, None
    if want_cpu:
        import oracle
        if oracle.ref_available():
            graphs = [(n, s, d) for (n, s, d) in pool]
            _, _, per_scc = oracle.ref_batch("scc", graphs, "seq")
            _, _, per_cc = oracle.ref_batch("cc", graphs, "seq")
            ref_svc = np.stack([np.array(per_scc), np.array(per_cc)], axis=1)
            ref_kind = "reference"
    sctx = gb.Context(device)
    # the merged runs take their size class's options (the committed table);
    # the one-at-a-time runs likewise
    from connectivity_gb300 import tune as gbtune
    gbtune.install(sctx)
    gbtune.install(ctx)
    # one warm-up stream through a server on the same context, so that
    # one-time costs (the memory pool's first growth, first launches) stay
    # out of the measured streams
    rng = np.random.default_rng(0)
    nwu = 1000
    wk = (rng.random(nwu) < 0.2).astype(np.int32)
    wi = rng.integers(0, pool_size, nwu)
    wu = gb.Server(sctx, budget_bytes=0, max_graphs=8192)
    wouts = [np.empty(pool[i][0], np.int32) for i in wi]
    for j in range(nwu):
        n, s, d = pool[wi[j]]
        wu.submit(int(wk[j]), n, s, d, arrival_ns=0, out=wouts[j])
    wu.start()
    wu.drain()
    wu.close()
    sweep = []
    for r_i, rate in enumerate(rates):
        rng = np.random.default_rng(1 + r_i)
        sat = rate == "max"
        cnt = 20000 if sat else int(max(200, float(rate) * seconds))
        kinds = (rng.random(cnt) < 0.2).astype(np.int32)
        idx = rng.integers(0, pool_size, cnt)
        if sat:
            arr = np.full(cnt, 0, np.int64)
        else:
            arr = (np.cumsum(rng.exponential(1e9 / float(rate), cnt)) + 2e6).astype(np.int64)
        outs = [np.empty(pool[i][0], np.int32) for i in idx]
        sv = gb.Server(sctx, budget_bytes=0, max_graphs=8192)
        for j in range(cnt):
            n, s, d = pool[idx[j]]
            sv.submit(int(kinds[j]), n, s, d, arrival_ns=int(arr[j]), out=outs[j])
        sv.start()
        sv.drain()
        st = sv.stats()
        sv.close()
        arr_s = arr / 1e9
        lat, fin = _fifo(arr_s, svc[idx, kinds])
        alone_gps = cnt / max(fin - arr_s[0], 1e-9)
        step = max(1, cnt // 100)
        same = all(np.array_equal(outs[j], alone(idx[j], kinds[j])) for j in range(0, cnt, step))
        e = {"rate": rate, "requests": cnt,
             "graphs_per_s": round(st.graphs_per_s, 1), "p50_ms": round(st.p50_ms, 3),
             "p99_ms": round(st.p99_ms, 3), "max_ms": round(st.max_ms, 3),
             "mean_merged": round(st.mean_batch, 1), "merged_runs": int(st.batches),
             "h2d_bytes": int(sum(pool[i][1].size * 8 for i in idx)),
             "d2h_bytes": int(sum(pool[i][0] * 4 for i in idx)),
             "gpu_one_at_a_time": {"graphs_per_s": round(alone_gps, 1),
                                   "p50_ms": round(float(np.median(lat)) * 1e3, 3),
                                   "p99_ms": round(float(np.quantile(lat, 0.99)) * 1e3, 3)},
             "speedup_vs_one_at_a_time": round(st.graphs_per_s / alone_gps, 2),
             "labels_equal_alone": bool(same), "labels_checked": len(range(0, cnt, step))}
        if ref_svc is not None:
            rl, rfin = _fifo(arr_s, ref_svc[idx, kinds])
            rgps = cnt / max(rfin - arr_s[0], 1e-9)
            e["cpu_baseline"] = {"graphs_per_s": round(rgps, 1),
                                 "p50_ms": round(float(np.median(rl)) * 1e3, 3),
                                 "p99_ms": round(float(np.quantile(rl, 0.99)) * 1e3, 3)}
            e["speedup_vs_cpu_baseline"] = round(st.graphs_per_s / rgps, 2)
        sweep.append(e)
    sctx.close()
    ctx.close()
    out = {
        "workload": (f"Poisson arrivals for {seconds:g} s per rate (at least 200 requests; 'max': "
                     "20,000 requests all arriving at t=0, the server's capacity), 80% SCC / 20% "
                     f"WCC, graphs drawn from a pool of {pool_size} of the batched size "
                     "distribution, edges in pinned host memory, labels to host; after a warm-up "
                     f"stream of {nwu:,} requests through a server on the same context"),
        "sweep": sweep,
        "max_sustained_graphs_per_s": max(e["graphs_per_s"] for e in sweep),
        "gpu_one_at_a_time_mean_service_ms": round(float(svc.mean()) * 1e3, 3),
    }
    if ref_svc is not None:
        out["cpu_baseline"] = {
            "kind": ref_kind, "cores": host_threads(),
            "how": ("each request served alone by the reference (run_scc or run_cc with all "
                    "host threads), first come first served, over the reference's measured "
                    "time for each pool graph (CSR build excluded, as in its timer)"),
            "mean_service_ms": round(float(ref_svc.mean()) * 1e3, 3)}
    return out


def headline(gb, ctx, stream, args, ws, rank, local, barrier, allmax):
    import numpy as np
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g = gb.Graph.rmat(ctx, args.scale, EF, SEED, ABC)
    graph_build_ms = (time.perf_counter() - t0) * 1e3
    # the hints freed and rebuilt three times: the median of the host's clock
    # around gb_graph_set_hints (allocation, launches, synchronise) and of
    # CUDA events on the library's stream around the same call
    hb_wall, hb_dev = [], []
    for _ in range(3):
        g.set_hints(ctx, False)
        h0 = torch.cuda.Event(enable_timing=True)
        h1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h0.record(stream)
        g.set_hints(ctx, True)
        h1.record(stream)
        h1.synchronize()
        hb_wall.append((time.perf_counter() - t0) * 1e3)
        hb_dev.append(h0.elapsed_time(h1))
    hint_build_ms = float(np.median(hb_wall))
    hint_build_dev_ms = float(np.median(hb_dev))
    n, m = g.n, g.m
    labels = torch.empty(n, dtype=torch.int32, device="cuda")
    o = gb.opts()

    W = max(args.warmup, 3)
    for _ in range(W):
        ctx.scc_async(g, labels.data_ptr(), o)
    ctx.sync()

    phys = local
    cvd = os.environ.get("CUDA_VISIBLE_DEVICES")
    if cvd:
        try:
            phys = int(cvd.split(",")[local])
        except ValueError:
            phys = local
    clocks = Clocks(phys)
    K = args.steps
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)  # first sample lands inside the timed region
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(K):
        ctx.scc_async(g, labels.data_ptr(), o)
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    barrier()
    ctx.sync()  # raises if any timed run failed on the device
    T = allmax(e0.elapsed_time(e1) / 1e3)
    phases = ctx.phase_times(min(K, 64))
    pm = phases.mean(axis=0)
    step_ms = T / K * 1e3
    value = job_gteps(m, ws, T, K)

    # the same steps without the hints
    g.set_hints(ctx, False)
    for _ in range(3):
        ctx.scc_async(g, labels.data_ptr(), o)
    ctx.sync()
    e0.record(stream)
    for _ in range(K):
        ctx.scc_async(g, labels.data_ptr(), o)
    e1.record(stream)
    torch.cuda.synchronize()
    ctx.sync()
    T_nh = allmax(e0.elapsed_time(e1) / 1e3)
    nh_labels = labels.cpu().numpy()
    g.set_hints(ctx, True)

    # the autotuner on this graph (its timed runs are outside the timed region)
    o_t, ms_t, ms_d = ctx.tune(g, 0, 3)
    from connectivity_gb300 import tune as gbtune
    autotuned = {"value": round(job_gteps(m, 1, ms_t / 1e3, 1), 3),
                 "defaults_value": round(job_gteps(m, 1, ms_d / 1e3, 1), 3),
                 "opts": gbtune.opts_to_dict(o_t),
                 "note": "device time of one run, best of 3, after the coordinate search"}

    # one more run with statistics (algorithmic bytes of each kernel)
    _, st = ctx.scc(g, labels=labels.data_ptr(), stats=True)
    gpu_labels = labels.cpu().numpy()

    # WCC of the same graph (run_cc on the mirrored graph: 2m arcs)
    wl = torch.empty(n, dtype=torch.int32, device="cuda")
    for _ in range(3):
        ctx.wcc_async(g, wl.data_ptr(), o)
    ctx.sync()
    e0.record(stream)
    for _ in range(K):
        ctx.wcc_async(g, wl.data_ptr(), o)
    e1.record(stream)
    torch.cuda.synchronize()
    ctx.sync()
    T_w = allmax(e0.elapsed_time(e1) / 1e3)
    wcc_labels = wl.cpu().numpy()
    del wl

    # e2e through the reference-shaped C ABI on pinned host buffers
    oo, oa, io, ia = g.to_host()
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
    odl, idl = pin(oo.astype(np.uint32)), pin(io.astype(np.uint32))
    oa_p, ia_p = pin(oa), pin(ia)
    out_p = pin(np.empty(n, np.int32))
    piv, avg = ctx.pivot(g, 0)
    gb.dropin_set_derive_share(E2E_SHARE)
    gb.run_scc_ref(n, oa_p, ia_p, odl, idl, piv, avg, 10000, out_p)  # warm-up
    KE = max(1, min(args.e2e_steps, K))
    barrier()
    t0 = time.perf_counter()
    for _ in range(KE):
        gb.run_scc_ref(n, oa_p, ia_p, odl, idl, piv, avg, 10000, out_p)
    TE = allmax(time.perf_counter() - t0)
    e2e_ok = bool(np.array_equal(out_p, gpu_labels))
    # gb_run_scc reads the out-CSR, both offset arrays and the part of
    # in_array it does not derive on the device
    e_split = int(idl[np.searchsorted(idl, E2E_SHARE * m, side="left")]) if m else 0
    h2d = (n + 1) * 4 * 2 + m * 4 + (m - e_split) * 4
    d2h = n * 4
    # the same calls at the two ends of the split: in-lists all copied, and
    # all derived on the device
    shares = {}
    for share in (0.0, 1.0):
        gb.dropin_set_derive_share(share)
        try:
            gb.run_scc_ref(n, oa_p, ia_p, odl, idl, piv, avg, 10000, out_p)  # warm-up
            barrier()
            t0 = time.perf_counter()
            for _ in range(KE):
                gb.run_scc_ref(n, oa_p, ia_p, odl, idl, piv, avg, 10000, out_p)
            ts = allmax(time.perf_counter() - t0)
            shares[share] = (ts, bool(np.array_equal(out_p, gpu_labels)))
        finally:
            gb.dropin_set_derive_share(E2E_SHARE)
    # the mirrored 32-bit CSR of cc's reader (per vertex: out- then
    # in-neighbours), for gb_run_cc
    odeg, ideg = np.diff(oo), np.diff(io)
    soff = np.zeros(n + 1, np.int64)
    np.cumsum(odeg + ideg, out=soff[1:])
    sadj = np.empty(2 * m, np.int32)
    sadj[np.repeat(soff[:-1] - oo[:-1], odeg) + np.arange(m)] = oa
    sadj[np.repeat(soff[:-1] + odeg - io[:-1], ideg) + np.arange(m)] = ia
    sdl, sadj_p = pin(soff.astype(np.uint32)), pin(sadj)
    # what gb_run_cc reads of it in place: the offsets, every vertex's first
    # entry, and the rest of the lists of the vertices outside the largest
    # component (the sampled union-find skips the others)
    sdeg = np.diff(soff)
    giant = np.bincount(wcc_labels).argmax() if n else 0
    cc_read = ((n + 1) * 4 + 4 * int(np.minimum(sdeg, 1).sum()) +
               4 * int(np.maximum(sdeg - 1, 0)[wcc_labels != giant].sum()))
    del sadj, soff, sdeg
    cout_p = pin(np.empty(n, np.int32))
    cpiv, cavg = ctx.pivot(g, 1)
    gb.run_cc_ref(n, sadj_p, sdl, cpiv, cavg, cout_p)  # warm-up
    barrier()
    t0 = time.perf_counter()
    for _ in range(KE):
        gb.run_cc_ref(n, sadj_p, sdl, cpiv, cavg, cout_p)
    TEW = allmax(time.perf_counter() - t0)
    e2e_wcc_ok = bool(np.array_equal(cout_p, wcc_labels))
    del sadj_p

    peak, peak_kind = peaks()
    # algorithmic bytes per launch, from the per-unit figures (O = 8 B per
    # int64 offset, I = 4 B per id or label):
    #   trim pass: 2*O*(n+1) + I*n + n/8
    #   traversal, per direction: O*(n+1) + I*m_visited + 2*n/8, plus per pull
    #   step O*(n+1), plus I per adjacency entry the pull steps scanned
    O, I = 8, 4
    trim8d = 2 * O * (n + 1) + I * n + n // 8
    dirs = (1 if st.fw_steps else 0) + (1 if st.bw_steps else 0)
    reach8d = (dirs * (O * (n + 1) + 2 * n // 8) + I * (st.m_visit_fw + st.m_visit_bw)
               + st.pull_steps * O * (n + 1) + I * st.pull_edges)

    def roof(kernel, nbytes, ms, touched):
        a = nbytes / (ms / 1e3) / 1e9
        return {"kernel": kernel, "achieved": round(a, 1), "frac": round(a / peak, 4),
                "algorithmic_bytes_per_launch": int(nbytes), "launch_ms": round(ms, 4),
                "touched_bytes_per_launch": int(touched),
                "touched_gbs": round(touched / (ms / 1e3) / 1e9, 1)}

    run_ms = float(pm[0] + pm[1] + pm[2])
    run8d = trim8d + reach8d + st.bytes_colour
    run = roof("k_run", run8d, run_ms, st.bytes_trim + st.bytes_reach + st.bytes_colour)
    phase_roofs = [
        dict(roof("trim", trim8d, float(pm[0]), st.bytes_trim), kernel="k_run: trim phase"),
        dict(roof("reach", reach8d, float(pm[1]), st.bytes_reach),
             kernel="k_run: reachability phase"),
        dict(roof("colour", st.bytes_colour, float(pm[2]), st.bytes_colour),
             kernel="k_run: colour phase (bytes touched)")]
    traffic = profile_traffic("k_run") if args.scale == SCALE else None
    pin_e = pins().get(f"rmat_s{args.scale}_ef{EF}_seed{SEED}", {})
    # the graph's edge list is its out-CSR read in order (sorted by source,
    # then target, as generated)
    src = np.repeat(np.arange(n, dtype=np.int32), odeg)
    parity = {
        "edges_digest_equal_reference_pin": (edge_digest(n, src, oa) == pin_e.get("edges")
                                             if pin_e else None),
        "scc_digest_equal_reference_pin": (label_digest(gpu_labels) == pin_e.get("scc_labels")
                                           if pin_e else None),
        "wcc_digest_equal_reference_pin": (label_digest(wcc_labels) == pin_e.get("cc_labels")
                                           if pin_e else None),
        "scc_verify_equal_reference_pin": (gb.scc_verify(gpu_labels) == pin_e.get("scc_verify")
                                           if pin_e else None),
        "wcc_verify_equal_reference_pin": (gb.cc_verify(wcc_labels) == pin_e.get("cc_verify")
                                           if pin_e else None),
        "no_hints_labels_equal": bool(np.array_equal(nh_labels, gpu_labels)),
        "scc_verify_line": gb.scc_verify(gpu_labels).strip(),
        "wcc_verify_line": gb.cc_verify(wcc_labels).strip(),
        "pin": "tests/golden/pins.json (the unmodified reference on the same edge list)",
    }
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GTEPS", "n_gpus": ws, "steps": K,
        "warmup": W, "ms_per_step": round(step_ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": config_for(n, m, args.scale, ws),
        "value_no_hints": round(job_gteps(m, ws, T_nh, K), 3),
        "ms_per_step_no_hints": round(T_nh / K * 1e3, 4),
        "graph_build_ms": round(graph_build_ms, 2),
        "graph_build_note": ("gb_graph_rmat: device R-MAT generation, radix-sort CSR (out and "
                             "in) and the hints, synchronous"),
        "hint_build_ms": round(hint_build_ms, 3),
        "hint_build_dev_ms": round(hint_build_dev_ms, 3),
        "hint_build_note": ("gb_graph_set_hints (both sides), median of 3 rebuilds: host clock "
                            "around the call, and CUDA events on the library's stream around it"),
        "e2e": {"value": round(job_gteps(m, ws, TE, KE), 3), "unit": "GTEPS",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": round(TE / KE * 1e3, 3), "steps": KE,
                "api": "gb_run_scc (run_scc signature, reference CSR layout, pinned host buffers; "
                       "builds no hints; the in-lists of the first derive_share of the in-edges "
                       "derived on the device from the out-CSR, the rest of in_array copied "
                       "beside them)",
                "labels_match_device_run": e2e_ok,
                "derive_share": E2E_SHARE,
                "by_share": {str(k): {"value": round(job_gteps(m, ws, v[0], KE), 3),
                                      "ms_per_step": round(v[0] / KE * 1e3, 3),
                                      "labels_match_device_run": v[1]}
                             for k, v in shares.items()}},
        "wcc": {"value": round(job_gteps(2 * m, ws, T_w, K), 3), "unit": "GTEPS (mirrored arcs)",
                "arcs": 2 * m, "ms_per_step": round(T_w / K * 1e3, 4), "steps": K,
                "api": "gb_wcc on the resident graph (out- and in-CSR walked as the mirrored "
                       "graph)",
                "e2e": {"value": round(job_gteps(2 * m, ws, TEW, KE), 3),
                        "unit": "GTEPS (mirrored arcs)",
                        "h2d_bytes_per_step": cc_read, "d2h_bytes_per_step": d2h,
                        "h2d_note": ("bytes of the pinned CSR the kernels read in place: the "
                                     "offsets, one entry per vertex and the lists of the "
                                     "vertices outside the largest component (the host link "
                                     "moves whole sectors); the CSR is "
                                     f"{(n + 1) * 4 + 2 * m * 4} bytes"),
                        "ms_per_step": round(TEW / KE * 1e3, 3), "steps": KE,
                        "api": "gb_run_cc (run_cc signature on cc's mirrored 32-bit CSR, pinned "
                               "host buffers; sampled union-find read in place)",
                        "labels_match_device_run": e2e_wcc_ok}},
        "parity": parity,
        "roofline": {"bound": "hbm",
                     "kernel": "k_run<1> (one cooperative launch per run: trim, reachability, "
                               "colour phases)",
                     "achieved": run["achieved"], "peak": peak, "unit": "GB/s",
                     "frac": run["frac"], "peak_source": f"{peak_kind} hbm_gbs (burst copy)",
                     "traffic": traffic,
                     "traffic_source": "profiles/traffic.json (ncu, one capture at scale 24)",
                     "dram_gbs_at_traffic": (round(traffic / (run_ms / 1e3) / 1e9, 1)
                                             if traffic else None),
                     "dram_frac_at_traffic": (round(traffic / (run_ms / 1e3) / 1e9 / peak, 4)
                                              if traffic else None),
                     "algorithmic_bytes_per_launch": run["algorithmic_bytes_per_launch"],
                     "launch_ms": run["launch_ms"],
                     "touched_bytes_per_launch": run["touched_bytes_per_launch"],
                     "units": {"n": n, "m": m, "m_visit_fw": st.m_visit_fw,
                               "m_visit_bw": st.m_visit_bw, "pull_steps": st.pull_steps,
                               "pull_edges_scanned": st.pull_edges},
                     "phases": phase_roofs},
        "autotuned": autotuned,
        "phases_ms": {k: round(float(v), 4) for k, v in
                      zip(("trim", "reach", "colour", "tail", "total"), pm)},
        "gpu_launches": 2 * K,
        "gpu_launches_note": "k_run (one cooperative launch) and the status latch per step",
        "clocks": ck,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        want, vline, tcpu, cores, tone, kind, what = cpu_scc_baseline(n, src, oa, args.cpu_reps)
        line["cpu_baseline"] = {
            "value": round(m / tcpu / 1e9, 4), "unit": "GTEPS", "cores": cores, "kind": kind,
            "sample": f"full workload, best of {args.cpu_reps} runs after 1 warm-up ({what})",
            "one_thread_value": round(m / tone / 1e9, 4),
            "host": {"nproc": os.cpu_count(), "machine": os.uname().machine}}
        parity["labels_equal_cpu_baseline"] = bool(np.array_equal(gpu_labels, want))
        parity["verify_equal_cpu_baseline"] = gb.scc_verify(gpu_labels) == vline
        wwant, wvline, twcc, wkind = cpu_cc_baseline(n, src, oa, args.cpu_reps)
        line["wcc"]["cpu_baseline"] = {
            "value": round(2 * m / twcc / 1e9, 4), "unit": "GTEPS (mirrored arcs)",
            "cores": cores, "kind": wkind,
            "sample": f"full workload, best of {args.cpu_reps} runs after 1 warm-up (run_cc)"}
        parity["wcc_labels_equal_cpu_baseline"] = bool(np.array_equal(wcc_labels, wwant))
        parity["wcc_verify_equal_cpu_baseline"] = gb.cc_verify(wcc_labels) == wvline
    g.close()
    return line


def run_gbconn(args):
    import torch

    import __graft_entry__
    if not os.path.exists(os.path.join(ROOT, "connectivity_gb300", "libgbconn.so")):
        __graft_entry__.build()
    import connectivity_gb300 as gb

    sections = set(x.strip() for x in args.sections.split(",") if x.strip())
    ws, rank, local = dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local))

    ctx = gb.Context(local)
    # a stream of our own: the library runs on it and the CUDA events are
    # recorded on it (torch's default stream is the legacy stream, handle 0,
    # which the library reads as "use the context's own stream")
    stream = torch.cuda.Stream(device=local)
    ctx.set_stream(stream.cuda_stream)
    line = headline(gb, ctx, stream, args, ws, rank, local, dist_barrier, dist_max)
    want_cpu = rank == 0 and ws == 1 and not args.no_cpu_baseline
    if "grid" in sections:
        line["grid"] = grid_section(gb, ctx, side=args.grid_side)
    if "batched" in sections:
        line["batched"] = batched_section(gb, ctx, stream, 5, args.batch_cpu_sample, want_cpu,
                                          ws, rank)
    ctx.close()
    if "served" in sections:
        rates = [r if r == "max" else float(r) for r in args.serve_rates.split(",") if r]
        line["served"] = served_section(gb, local, rates, args.serve_seconds, args.serve_pool,
                                        want_cpu)
        line["served"]["opts"] = "size-class table (connectivity_gb300/tables/classes_scc.json)"
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as tdist
        tdist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gbconn(args)


if __name__ == "__main__":
    main()
