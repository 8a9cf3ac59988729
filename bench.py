#!/usr/bin/env python
"""Benchmark of the GB300 k-core peel (one JSON line on rank 0).

Default workload: the single-graph R-MAT scale-20 edge-factor-5 peel (1,048,576
vertices, 5,242,880 directed draws, a/b/c/d = .57/.19/.19/.05, seed 2),
symmetrised and deduplicated, uint32 CSR resident in HBM.  A step is one full
peel of that graph (every level until all vertices are peeled).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config 1|2|3] [--impl ours|reference]

--impl reference times the reference algorithm's CPU restatement (the
level-synchronous peel of src/ours.cc:117-160, oracle/kc_oracle.c) on all host
cores; the reference has no CPU peel of its own.  Multi-GPU runs are replicas
(one independent graph per rank, no collective on the data path).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import platform
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "k-core edges/s & HBM GB/s; batched graphs/s, p50/p99 latency vs plain peel"
L2_FLUSH_BYTES = 512 << 20   # > 129 MB L2

# DRAM bytes (read + write) of one peel -- the persistent kernel plus the
# one-CTA tail kernel it hands the last levels to -- from one ncu capture of
# the same workload (profiles/peel_persistent_rmat-s20-ef5.md); None where not
# captured.
NCU_TRAFFIC = {2: 45_338_880 + 3_630_080 + 7_795_712 + 0}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        self.rows = []
        if self.p is None:
            return
        time.sleep(0.25)
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 7:
                self.rows.append(f)

    def summary(self) -> dict:
        if not getattr(self, "rows", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if "Active" in r[3 + i]
                          and "Not" not in r[3 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(self.rows)}


def measured_peak_hbm() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def cpu_model() -> str:
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def reference_arm(args, rank, world):
    """The reference algorithm on the host cores (CPU restatement, all threads)."""
    if rank != 0:
        return
    if args.config in (4, 5):
        return reference_arm_graphs(args, world)
    from kcoregpu_gb300 import workloads as W
    from oracle import kc_oracle as O
    off, nbr = W.single_graph(args.config)
    m = len(nbr) // 2
    nth = os.cpu_count() or 1
    for _ in range(args.warmup):
        O.levelsync(off, nbr, nthreads=nth)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, kmax, levels = O.levelsync(off, nbr, nthreads=nth)
        times.append(time.perf_counter() - t0)
    t = sum(times) / len(times)
    val = m / t
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": val, "unit": "edges/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": W.SINGLE[args.config]["name"], "V": len(off) - 1, "undirected_edges": m,
                   "kmax": kmax, "levels": levels},
        "cpu_baseline": {"value": val, "unit": "edges/s", "cores": nth, "kind": "port",
                         "sample": f"full graph x {args.steps} peels (level-synchronous restatement of "
                                   f"src/ours.cc:117-160, OpenMP, {cpu_model()})"},
        "e2e": {"value": val, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def reference_arm_graphs(args, world, sample: int = 48):
    """Batched / served workloads on the host cores: the level-synchronous
    restatement (all threads) over a bounded sample of the workload's graphs
    (the first `sample` graphs of the batch, or requests of the stream),
    reported as graphs/s."""
    from kcoregpu_gb300 import workloads as W
    from oracle import kc_oracle as O
    nth = os.cpu_count() or 1
    if args.config == 4:
        seg = W.batch(sample)
        graphs = [seg.graph(g) for g in range(seg.ngraphs)]
        name, what = W.BATCH["name"], f"graphs 0..{sample - 1} of the batch"
    else:
        graphs = [W.served_request(i) for i in range(sample)]
        name, what = W.SERVED["name"], f"requests 0..{sample - 1} of the stream (no scale-24 graph)"
    for off, nbr in graphs[: max(1, args.warmup)]:
        O.levelsync(off, nbr, nthreads=nth)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for off, nbr in graphs:
            O.levelsync(off, nbr, nthreads=nth)
        times.append(time.perf_counter() - t0)
    t = sum(times) / len(times)
    val = len(graphs) / t
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": val, "unit": "graphs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": name, "sample_graphs": len(graphs)},
        "cpu_baseline": {"value": val, "unit": "graphs/s", "cores": nth, "kind": "port",
                         "sample": f"{what}, level-synchronous restatement of src/ours.cc:117-160, "
                                   f"OpenMP, {cpu_model()}"},
        "e2e": {"value": val, "unit": "graphs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def max_over_ranks(values, world: int, device="cpu"):
    """Element-wise maximum of per-rank timings (all_reduce MAX) -> list."""
    if world <= 1:
        return list(values)
    import torch
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return t.tolist()


def cpu_baseline(off, nbr):
    """The project's single-thread BZ bucket peel timed on the same CSR."""
    from oracle import kc_oracle as O
    m = len(nbr) // 2
    reps, t_tot = 0, 0.0
    while t_tot < 3.0 and reps < 50:
        t0 = time.perf_counter()
        O.bz(off, nbr)
        t_tot += time.perf_counter() - t0
        reps += 1
    return {"value": m * reps / t_tot, "unit": "edges/s", "cores": 1, "kind": "port",
            "sample": f"full graph x {reps} Batagelj-Zaversnik peels, single thread ({cpu_model()}, "
                      f"{os.cpu_count()} cores on host)"}


def reference_gpu(off, nbr, tmpdir: Path):
    """The reference's own GPU kernels (src/ours.cc, unmodified cubin) with its
    host loop replayed; None when the prebuilt cubin is absent."""
    cubin = ROOT / "oracle" / "_ref" / "ref_peel.cubin"
    drv = ROOT / "oracle" / "_build" / "ref_peel_driver"
    if not cubin.exists() or not drv.exists():
        return None
    tmpdir.mkdir(parents=True, exist_ok=True)
    f = tmpdir / "csr.bin"
    with open(f, "wb") as fh:
        np.array([len(off) - 1, len(nbr)], np.uint32).tofile(fh)
        off.tofile(fh)
        nbr.tofile(fh)
    out = tmpdir / "core.bin"
    r = subprocess.run([str(drv), str(cubin), str(f), str(out)], capture_output=True, text=True,
                       timeout=300)
    if r.returncode != 0:
        return {"unavailable": (r.stderr or r.stdout).strip()[:200]}
    tok = r.stdout.split()
    ms = float(tok[tok.index("ms") + 1])
    return {"ms": ms, "edges_per_s": (len(nbr) // 2) / (ms / 1e3),
            "kmax": int(tok[tok.index("kmax") + 1]),
            "core": np.fromfile(out, dtype=np.uint32)}


def e2e_leg(args, kc, V: int, arcs: int, off, nbr, want, flush, torch) -> float:
    """End to end through the public one-shot call (kc_peel_csr): pinned H2D of
    the CSR, the device-side CSR check, the peel and D2H of the core numbers,
    every step; returns the mean seconds per call."""
    lib = kc.lib()
    h_off = lib.kc_host_alloc(4 * (V + 1))
    h_nbr = lib.kc_host_alloc(4 * max(arcs, 1))
    h_core = lib.kc_host_alloc(4 * max(V, 1))
    a_off = np.ctypeslib.as_array(C.cast(h_off, C.POINTER(C.c_uint32)), shape=(V + 1,))
    a_nbr = np.ctypeslib.as_array(C.cast(h_nbr, C.POINTER(C.c_uint32)), shape=(max(arcs, 1),))
    a_off[:] = off
    a_nbr[:arcs] = nbr
    u32p = C.POINTER(C.c_uint32)
    kout = C.c_uint32()

    def e2e_call():
        rc = lib.kc_peel_csr(C.cast(h_off, u32p), C.cast(h_nbr, u32p), V, C.cast(h_core, u32p), C.byref(kout))
        if rc:
            raise SystemExit(f"kc_peel_csr failed: {rc}")

    for _ in range(max(1, args.warmup)):
        e2e_call()
    e2e_t = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_call()
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = sum(e2e_t) / len(e2e_t)
    got = np.ctypeslib.as_array(C.cast(h_core, u32p), shape=(V,))
    if not np.array_equal(got, want):
        raise SystemExit("bench: e2e core numbers differ from the oracle")
    for p in (h_off, h_nbr, h_core):
        lib.kc_host_free(p)
    return e2e_s


def batched_leg(args, torch, flush, with_cpu: bool, with_baseline: bool = True, ngraphs: int | None = None):
    """The batched workload (4,096 graphs in one persistent launch): graphs/s,
    the plain one-graph-per-launch peel beside it, and the CPU bucket peel over
    all host cores.  ngraphs < 4,096 takes the first graphs only (the small
    case profiled by ncu)."""
    from kcoregpu_gb300 import batch as B
    from kcoregpu_gb300 import workloads as W
    from oracle import kc_oracle as O
    t0 = time.perf_counter()
    seg = W.batch(ngraphs)
    gen_s = time.perf_counter() - t0
    G, Vt, At = seg.ngraphs, int(seg.vbase[-1]), int(seg.abase[-1])
    stream = torch.cuda.Stream()
    b = B.Batch(seg)
    b.set_stream(stream.cuda_stream)
    core, kmax, _ = b.peel()
    t0 = time.perf_counter()
    want, wk = O.batch_bz(seg.vbase, seg.abase, seg.offsets, seg.neighbors, O.num_threads())
    cpu_s = time.perf_counter() - t0
    if not (np.array_equal(core, want) and np.array_equal(kmax, wk)):
        raise SystemExit("bench: batched core numbers differ from the oracle")
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            b.peel_async()
        ms = []
        for _ in range(args.steps):
            flush.zero_()
            b.peel_async()
            ms.append(b.fetch(want_core=False)[2]["peel_ms"])
    step_ms = sum(ms) / len(ms)
    per_graph_ms = b.peel_per_graph() if with_baseline else None
    B_alg = W.batch_algorithmic_bytes(seg, kmax)
    peak, _ = measured_peak_hbm()
    out = {"workload": W.BATCH["name"], "graphs": G, "V": Vt, "arcs": At, "generation_s": gen_s,
           "graphs_per_s": G / (step_ms / 1e3), "ms_per_step": step_ms,
           "edges_per_s": (At // 2) / (step_ms / 1e3), "hbm_gbs": B_alg / (step_ms / 1e3) / 1e9,
           "roofline_frac": B_alg / (step_ms / 1e3) / 1e9 / peak, "algorithmic_bytes": B_alg,
           "plan": {k: v for k, v in b.plan().items() if k != "schedule"},
           "kmax_max": int(kmax.max())}
    if per_graph_ms is not None:
        out["plain_per_graph"] = {"ms": per_graph_ms, "graphs_per_s": G / (per_graph_ms / 1e3),
                                  "speedup_of_batched": per_graph_ms / step_ms}
    if with_cpu:
        out["cpu_baseline"] = {"value": G / cpu_s, "unit": "graphs/s", "cores": O.num_threads(),
                               "kind": "port", "sample": "all 4,096 graphs, one Batagelj-Zaversnik per graph, "
                                                         "OpenMP over graphs"}
    b.free()
    return out


def served_leg(requests: int, mmax: int | None, with_big: bool, rates, seed: int = 5):
    """Continuous batching: a seeded Poisson stream of requests submitted to the
    server at each arrival rate (and all at once for saturation); latency is
    submit -> core numbers on the host.  The plain one-graph-at-a-time peel
    (kc_peel_csr per request, upload and download included) runs the same
    stream for comparison."""
    import kcoregpu_gb300 as kc
    from kcoregpu_gb300 import workloads as W
    from kcoregpu_gb300.serve import Server
    t0 = time.perf_counter()
    reqs = [W.served_request(i, mmax=mmax) for i in range(requests)]
    big_pos = None
    if with_big:
        big_pos = requests // 2
        reqs.insert(big_pos, W.served_big())
    gen_s = time.perf_counter() - t0
    edges = [len(n) // 2 for _, n in reqs]
    srv = Server()
    srv.wait(srv.submit(*reqs[0]))   # warm-up (kernel launch, pool growth)
    if big_pos is not None:          # and the big graph's own pool growth and first device touch
        srv.wait(srv.submit(*reqs[big_pos]))
    rng = np.random.default_rng(seed)
    sweep = []
    for rate in list(rates) + [None]:
        gaps = rng.exponential(1.0 / rate, len(reqs)) if rate else np.zeros(len(reqs))
        arrive = np.cumsum(gaps) - gaps[0]
        ids = []
        start = time.perf_counter()
        for a, (o, n) in zip(arrive, reqs):
            while time.perf_counter() - start < a:
                time.sleep(min(0.0005, max(0.0, a - (time.perf_counter() - start))))
            ids.append(srv.submit(o, n))
        res = [srv.wait(r, timeout_s=300) for r in ids]
        span = time.perf_counter() - start
        lat = np.array([t["latency_us"] for _, _, t in res]) / 1e3
        pt = {"rate": rate or "all-at-once", "graphs_per_s": len(reqs) / span, "edges_per_s": sum(edges) / span,
              "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
              "max_gang": max(t["gang"] for _, _, t in res)}
        if big_pos is not None:
            pt["big_graph_latency_ms"] = float(lat[big_pos])
        sweep.append(pt)
    st = srv.stats()
    srv.close()
    # the same warm-up as the server's: the first call and the big graph's
    # first call grow the one-shot path's device buffers
    kc.peel_csr(*reqs[0])
    if big_pos is not None:
        kc.peel_csr(*reqs[big_pos])
    t1 = time.perf_counter()
    for o, n in reqs:
        kc.peel_csr(o, n)
    plain_s = time.perf_counter() - t1
    sat = sweep[-1]
    return {"workload": W.SERVED["name"] if with_big else f"served-{requests}-requests-m<= {mmax}",
            "requests": len(reqs), "undirected_edges": int(sum(edges)), "generation_s": gen_s,
            "sweep": sweep, "saturated_graphs_per_s": sat["graphs_per_s"],
            "plain_one_at_a_time": {"graphs_per_s": len(reqs) / plain_s, "seconds": plain_s,
                                    "speedup_of_served": sat["graphs_per_s"] / (len(reqs) / plain_s)},
            "peak_device_bytes": st["peak_in_use"], "blocks": st["blocks"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--config", type=int, default=2, choices=[1, 2, 3, 4, 5])
    ap.add_argument("--no-serve", action="store_true", help="skip the served leg of the default run")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched leg of the default run")
    ap.add_argument("--graphs", type=int, default=None,
                    help="--config 4: the first N graphs of the batch only (a small case for ncu)")
    ap.add_argument("--profile", action="store_true",
                    help="device legs only (no e2e, CPU or reference-GPU legs): the command profiled by ncu")
    ap.add_argument("--profile-e2e", action="store_true",
                    help="--config 1-3: the one-shot end-to-end leg alone (upload, device-side CSR check, "
                         "peel, download): the command profiled by ncu for the CSR check")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return reference_arm(args, rank, world)

    import torch
    import kcoregpu_gb300 as kc
    from kcoregpu_gb300 import workloads as W
    from oracle import kc_oracle as O

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    if args.config == 5:
        barrier()
        with Clocks(local) as clk:
            sv = served_leg(W_requests := 120, None, True, rates=[25, 50, 100, 200, 400, 800])
        barrier()
        if rank == 0:
            sat = sv["sweep"][-1]
            line = {"metric": METRIC, "value": world * sv["saturated_graphs_per_s"], "unit": "graphs/s",
                    "n_gpus": world, "steps": W_requests, "warmup": 1, "ms_per_step": 1e3 / sv["saturated_graphs_per_s"],
                    "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
                    "data": "synthetic", "config": {"workload": sv["workload"], "requests": sv["requests"],
                                                    "undirected_edges": sv["undirected_edges"],
                                                    "inputs": "host memory, uploaded per request"},
                    "p50_ms": sat["p50_ms"], "p99_ms": sat["p99_ms"],
                    "e2e": {"value": world * sv["saturated_graphs_per_s"], "unit": "graphs/s",
                            "note": "every request's upload and result download are inside its latency"},
                    "clocks": clk.summary(), "served": sv}
            print(json.dumps(line), flush=True)
        return

    if args.config == 4:
        flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
        barrier()
        with Clocks(local) as clk:
            bl = batched_leg(args, torch, flush, with_cpu=not (args.no_cpu or args.profile),
                             with_baseline=not args.profile, ngraphs=args.graphs)
        barrier()
        if args.profile:
            if rank == 0:
                print(json.dumps({"profile_run": True, "ms_per_step": bl["ms_per_step"], "graphs": bl["graphs"],
                                  "workload": bl["workload"]}), flush=True)
            return
        if rank == 0:
            line = {"metric": METRIC, "value": world * bl["graphs_per_s"], "unit": "graphs/s", "n_gpus": world,
                    "steps": args.steps, "warmup": args.warmup, "ms_per_step": bl["ms_per_step"],
                    "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
                    "data": "synthetic", "config": {"workload": bl["workload"], "graphs": bl["graphs"],
                                                    "V": bl["V"], "arcs": bl["arcs"],
                                                    "l2": "flushed between timed steps (512 MiB write)",
                                                    "inputs": "resident in HBM"},
                    "roofline": {"bound": "hbm", "achieved": bl["hbm_gbs"], "peak": measured_peak_hbm()[0],
                                 "unit": "GB/s", "frac": bl["roofline_frac"], "traffic": None,
                                 "algorithmic_bytes": bl["algorithmic_bytes"]},
                    "gpu_launches": args.steps, "clocks": clk.summary(), "batched": bl}
            if "cpu_baseline" in bl:
                line["cpu_baseline"] = bl["cpu_baseline"]
            print(json.dumps(line), flush=True)
        return

    off, nbr = W.single_graph(args.config)
    V, arcs = len(off) - 1, len(nbr)
    m = arcs // 2
    stream = torch.cuda.Stream()
    g = kc.DeviceGraph(off, nbr)
    g.set_stream(stream.cuda_stream)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")

    # correctness of the benchmarked graph (untimed)
    core, kmax, st0 = g.peel()
    want, wk = O.bz(off, nbr)
    if not (np.array_equal(core, want) and kmax == wk):
        raise SystemExit("bench: GPU core numbers differ from the oracle")

    if args.profile_e2e:
        e2e_ms = e2e_leg(args, kc, V, arcs, off, nbr, want, flush, torch) * 1e3
        if rank == 0:
            print(json.dumps({"profile_run": True, "e2e_ms": e2e_ms, "workload": W.SINGLE[args.config]["name"]}),
                  flush=True)
        return

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            g.peel_async()
        stream.synchronize()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        kern_ms = []
        barrier()
        torch.cuda.synchronize()
        with Clocks(local) as clk:
            t_wall = time.perf_counter()
            for i in range(args.steps):
                flush.zero_()                   # L2 flushed between timed steps
                starts[i].record(stream)
                g.peel_async()
                ends[i].record(stream)
                _, _, st = g.fetch(want_core=False)   # kernel-only time from the library's events
                kern_ms.append(st["peel_ms"])
            torch.cuda.synchronize()
            t_wall = time.perf_counter() - t_wall
        barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = sum(step_ms) / len(step_ms)
    kms = sum(kern_ms) / len(kern_ms)
    ms, kms = max_over_ranks([ms, kms], world, device="cuda")

    if args.profile:
        if rank == 0:
            print(json.dumps({"profile_run": True, "ms_per_step": ms, "kernel_ms": kms,
                              "workload": W.SINGLE[args.config]["name"]}), flush=True)
        return

    e2e_s = e2e_leg(args, kc, V, arcs, off, nbr, want, flush, torch)

    if rank != 0:
        return
    peak, peak_kind = measured_peak_hbm()
    B = W.algorithmic_bytes(V, arcs, kmax)
    achieved = B / (kms / 1e3) / 1e9
    value = world * m / (ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": "edges/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": W.SINGLE[args.config]["name"], "V": V, "undirected_edges": m, "arcs": arcs,
                   "kmax": kmax, "levels": kmax + 1, "parallelism": f"replicas{world}",
                   "l2": "flushed between timed steps (512 MiB write)", "inputs": "resident in HBM"},
        "hbm_gbs": achieved, "arcs_per_s": world * arcs / (ms / 1e3),
        "kernel_ms": kms,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind + " hbm_gbs",
                     "algorithmic_bytes": B,
                     "traffic": NCU_TRAFFIC.get(args.config)},
        "e2e": {"value": world * m / e2e_s, "unit": "edges/s", "ms": e2e_s * 1e3,
                "h2d_bytes_per_step": 4 * (V + 1) + 4 * arcs, "d2h_bytes_per_step": 4 * V},
        "gpu_launches": 2 * args.steps,   # persistent peel + tail kernel per step
        "clocks": clk.summary(),
        "wall_s": t_wall,
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(off, nbr)
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        ref = reference_gpu(off, nbr, Path(td))
        if ref is not None and "core" in ref:
            ref["bit_exact_vs_oracle"] = bool(np.array_equal(ref.pop("core"), want))
    if ref is not None:
        line["reference_gpu"] = ref
    if not args.no_batch:
        try:
            bl = batched_leg(argparse.Namespace(steps=3, warmup=1), torch, flush, with_cpu=not args.no_cpu)
            line["batched"] = bl
        except Exception as e:   # the single-graph line stands on its own
            line["batched"] = {"error": repr(e)[:200]}
    if not args.no_serve:
        try:   # a reduced sample of the served stream (the full one is --config 5)
            line["served_sample"] = served_leg(60, 2_000_000, False, rates=[200, 800])
        except Exception as e:
            line["served_sample"] = {"error": repr(e)[:200]}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
