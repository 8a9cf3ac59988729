#!/usr/bin/env python
"""Benchmark of the GB300 k-core peel (one JSON line on rank 0).

Headline workload (default): the single-graph peel of the skewed Chung-Lu
graph (2,400,000 vertices, 5,000,000 undirected edges, degree exponent 2.1,
max expected degree 100,000, seed 3), uint32 CSR resident in HBM.  A step is
one full peel of that graph (every level until all vertices are peeled).  The
same line carries, as sub-records with their own roofline, the two R-MAT
single-graph workloads (400K vertices / 3.4M draws, and scale 20 edge factor
5), the batched workload (4,096 graphs in one persistent launch) and the
served workload (a Poisson stream of 120 requests plus the R-MAT scale-24
edge-factor-16 graph, every result checked against the CPU oracle).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config 1|2|3|4|5] [--impl ours|reference]

--impl reference times the reference algorithm's CPU restatement (the
level-synchronous peel of src/ours.cc:117-160, oracle/kc_oracle.c) on all host
cores, on input graphs built by the oracle's own generators: that arm loads no
library of the product.  Multi-GPU runs are replicas (one independent graph per
rank, no collective on the data path).
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
TIMING_NOTE = ("GPU arm: L2 flushed between timed steps (512 MiB write), inputs resident in HBM; "
               "reference arm: host memory")

# DRAM bytes (read + write) of one peel per workload, from one ncu capture of
# that workload with the build that is measured here: the h-index kernel, the
# cluster kernel it hands its last iterations to, plus the level peel's
# persistent and tail kernels (which return at once after it), and, for the
# level peel method, its persistent and one-CTA tail kernels.
NCU_TRAFFIC = {1: 30_764_800 + 712_192 + 7_332_352 + 65_792 + 29_184,
               2: 63_110_144 + 10_822_656 + 839_424 + 66_816 + 29_184,
               3: 84_662_016 + 25_049_088 + 1_640_704 + 65_536 + 28_928}
NCU_TRAFFIC_LEVEL_PEEL = {1: 27_792_896 + 837_120 + 11_156_224, 2: 45_363_200 + 3_072_768 + 6_451_968 + 4_608,
                          3: 51_795_968 + 6_880_512 + 5_824_256}


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


def single_config(cfg: int, V: int, arcs: int, kmax: int) -> dict:
    """The `config` of a single-graph line; both arms print the same one."""
    from kcoregpu_gb300 import workloads as W
    return {"workload": W.SINGLE[cfg]["name"], "V": V, "undirected_edges": arcs // 2, "arcs": arcs,
            "kmax": kmax, "levels": kmax + 1, "timing": TIMING_NOTE}


def graphs_config(cfg: int) -> dict:
    """The `config` of a batched or served line; both arms print the same one."""
    from kcoregpu_gb300 import workloads as W
    if cfg == 4:
        return {"workload": W.BATCH["name"], "graphs": W.BATCH["ngraphs"], "timing": TIMING_NOTE}
    return {"workload": W.SERVED["name"], "requests": SERVED_REQUESTS + 1, "timing": TIMING_NOTE}


SERVED_REQUESTS = 120
SERVED_RATES = [25, 50, 100, 200, 400, 800]


def reference_arm(args, rank, world):
    """The reference algorithm on the host cores (CPU restatement, all
    threads), on inputs from the oracle's generators."""
    if rank != 0:
        return
    if args.config in (4, 5):
        return reference_arm_graphs(args, world)
    from oracle import kc_oracle as O
    from oracle import kc_workloads as OW
    off, nbr = OW.single_graph(args.config)
    V, arcs = len(off) - 1, len(nbr)
    m = arcs // 2
    nth = os.cpu_count() or 1
    for _ in range(args.warmup):
        O.levelsync(off, nbr, nthreads=nth)
    times = []
    kmax = levels = 0
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
        "config": single_config(args.config, V, arcs, kmax),
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
    from oracle import kc_oracle as O
    from oracle import kc_workloads as OW
    nth = os.cpu_count() or 1
    if args.config == 4:
        seg = OW.batch(sample)
        graphs = [seg.graph(g) for g in range(seg.ngraphs)]
        what = f"graphs 0..{sample - 1} of the batch"
    else:
        graphs = [OW.served_request(i) for i in range(sample)]
        what = f"requests 0..{sample - 1} of the stream (no scale-24 graph)"
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
        "config": graphs_config(args.config),
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


def single_leg(cfg: int, args, torch, flush, local: int, world: int, steps: int, warmup: int,
               full: bool = True) -> dict:
    """One single-graph workload: the device-timed peel (value), its roofline,
    and -- with `full` -- the e2e call, the CPU BZ and the reference's own
    GPU kernels beside it."""
    import kcoregpu_gb300 as kc
    from kcoregpu_gb300 import workloads as W
    from oracle import kc_oracle as O
    off, nbr = W.single_graph(cfg)
    V, arcs = len(off) - 1, len(nbr)
    m = arcs // 2
    stream = torch.cuda.Stream()
    g = kc.DeviceGraph(off, nbr)
    g.set_stream(stream.cuda_stream)

    # correctness of the benchmarked graph (untimed)
    core, kmax, st0 = g.peel()
    want, wk = O.bz(off, nbr)
    if not (np.array_equal(core, want) and kmax == wk):
        raise SystemExit(f"bench: GPU core numbers differ from the oracle on {W.SINGLE[cfg]['name']}")

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    with torch.cuda.stream(stream):
        for _ in range(warmup):
            flush.zero_()
            g.peel_async()
        stream.synchronize()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        kern_ms = []
        barrier()
        torch.cuda.synchronize()
        with Clocks(local) as clk:
            t_wall = time.perf_counter()
            for i in range(steps):
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
    peak, peak_kind = measured_peak_hbm()
    B = W.algorithmic_bytes(V, arcs, kmax)
    achieved = B / (kms / 1e3) / 1e9
    rec = {"workload": W.SINGLE[cfg]["name"], "config": single_config(cfg, V, arcs, kmax),
           "steps": steps, "warmup": warmup, "ms_per_step": ms, "kernel_ms": kms,
           "edges_per_s": world * m / (ms / 1e3), "arcs_per_s": world * arcs / (ms / 1e3),
           "hbm_gbs": achieved,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "peak_kind": peak_kind + " hbm_gbs",
                        "algorithmic_bytes": B,
                        "traffic": (NCU_TRAFFIC if st0["method"] == 1 else NCU_TRAFFIC_LEVEL_PEEL).get(cfg)},
           "method": "hindex" if st0["method"] == 1 else "level peel", "iterations": st0["iterations"],
           # per step: the h-index kernel and the cluster kernel it hands its
           # last iterations to (h-index method; the cluster kernel is not
           # launched with KC_HX_HANDOFF=0), the persistent peel kernel and the
           # tail kernel (both return at once after an h-index peel that
           # converged)
           "gpu_launches": ((3 + (os.environ.get("KC_HX_HANDOFF", "1") != "0")) if st0["method"] == 1 else 2) * steps,
           "clocks": clk.summary(), "wall_s": t_wall, "bit_exact_vs_oracle": True}
    if args.profile:
        g.free()
        return rec
    if full:
        e2e_s = e2e_leg(argparse.Namespace(steps=steps, warmup=warmup), kc, V, arcs, off, nbr, want, flush, torch)
        rec["e2e"] = {"value": world * m / e2e_s, "unit": "edges/s", "ms": e2e_s * 1e3,
                      "h2d_bytes_per_step": 4 * (V + 1) + 4 * arcs, "d2h_bytes_per_step": 4 * V}
        if not args.no_cpu:
            rec["cpu_baseline"] = cpu_baseline(off, nbr)
        import tempfile
        with tempfile.TemporaryDirectory() as td:
            ref = reference_gpu(off, nbr, Path(td))
            if ref is not None and "core" in ref:
                ref["bit_exact_vs_oracle"] = bool(np.array_equal(ref.pop("core"), want))
        if ref is not None:
            rec["reference_gpu"] = ref
    g.free()
    return rec


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
           "graphs_per_s": G / (step_ms / 1e3), "ms_per_step": step_ms, "steps": args.steps,
           "edges_per_s": (At // 2) / (step_ms / 1e3), "hbm_gbs": B_alg / (step_ms / 1e3) / 1e9,
           "roofline_frac": B_alg / (step_ms / 1e3) / 1e9 / peak, "algorithmic_bytes": B_alg,
           "plan": {k: v for k, v in b.plan().items() if k != "schedule"},
           "kmax_max": int(kmax.max()), "bit_exact_vs_oracle": True}
    if per_graph_ms is not None:
        out["plain_per_graph"] = {"ms": per_graph_ms, "graphs_per_s": G / (per_graph_ms / 1e3),
                                  "speedup_of_batched": per_graph_ms / step_ms}
    if with_cpu:
        out["cpu_baseline"] = {"value": G / cpu_s, "unit": "graphs/s", "cores": O.num_threads(),
                               "kind": "port", "sample": f"all {G:,} graphs, one Batagelj-Zaversnik per graph, "
                                                         "OpenMP over graphs"}
    b.free()
    return out


def _oracle_all(graphs):
    """BZ core numbers and kmax of every graph, on all host cores (the calls
    release the GIL)."""
    import concurrent.futures as cf
    from oracle import kc_oracle as O
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        return list(ex.map(lambda g: O.bz(*g), graphs))


def served_leg(requests: int, mmax: int | None, with_big: bool, rates, seed: int = 5, saturated_passes: int = 3):
    """Continuous batching: a seeded Poisson stream of requests submitted to the
    server at each arrival rate, then all at once (saturation) in
    `saturated_passes` back-to-back passes; latency is submit -> core numbers
    on the host.  Every result of every pass is compared with the CPU BZ peel.
    The plain one-graph-at-a-time peel (kc_peel_csr per request, upload and
    download included) runs the same stream for comparison."""
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
    t0 = time.perf_counter()
    wants = _oracle_all(reqs)
    oracle_s = time.perf_counter() - t0
    edges = [len(n) // 2 for _, n in reqs]
    mismatches = 0
    checked = 0

    def check(res):
        nonlocal mismatches, checked
        for (core, kmax, _), (wc, wk) in zip(res, wants):
            checked += 1
            if kmax != wk or not np.array_equal(core, wc):
                mismatches += 1

    srv = Server()
    srv.wait(srv.submit(*reqs[0]))   # warm-up (kernel launch, pool growth)
    if big_pos is not None:          # and the big graph's own pool growth and first device touch
        srv.wait(srv.submit(*reqs[big_pos]))
    rng = np.random.default_rng(seed)
    sweep = []
    for rate in list(rates) + [None] * saturated_passes:
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
        check(res)
        lat = np.array([t["latency_us"] for _, _, t in res]) / 1e3
        pt = {"rate": rate or "all-at-once", "graphs_per_s": len(reqs) / span, "edges_per_s": sum(edges) / span,
              "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
              "max_gang": max(t["gang"] for _, _, t in res)}
        if big_pos is not None:
            pt["big_graph_latency_ms"] = float(lat[big_pos])
            bt = res[big_pos][2]
            pt["big_graph_peel_ms"] = bt["peel_us"] / 1e3
            pt["big_graph_parts_ms"] = {"queue": bt["queue_us"] / 1e3, "copy_in": bt["copy_in_us"] / 1e3,
                                        "copy_out": bt["copy_out_us"] / 1e3}
        sweep.append(pt)
        del res
    st = srv.stats()
    srv.close()
    # the same warm-up as the server's: the first call and the big graph's
    # first call grow the one-shot path's device buffers
    kc.peel_csr(*reqs[0])
    if big_pos is not None:
        kc.peel_csr(*reqs[big_pos])
    t1 = time.perf_counter()
    plain = [kc.peel_csr(o, n) for o, n in reqs]
    plain_s = time.perf_counter() - t1
    plain_bad = sum(1 for (c, k), (wc, wk) in zip(plain, wants) if k != wk or not np.array_equal(c, wc))
    sat = sweep[-saturated_passes:]
    gps = [p["graphs_per_s"] for p in sat]
    p50 = [p["p50_ms"] for p in sat]
    p99 = [p["p99_ms"] for p in sat]
    return {"workload": W.SERVED["name"] if with_big else f"served-{requests}-requests-m<= {mmax}",
            "requests": len(reqs), "undirected_edges": int(sum(edges)), "generation_s": gen_s,
            "oracle_s": oracle_s, "sweep": sweep,
            "saturated_graphs_per_s": statistics.median(gps),
            "saturated_passes": {"graphs_per_s": gps, "p50_ms": p50, "p99_ms": p99,
                                 "p50_spread": max(p50) / min(p50) if min(p50) > 0 else None,
                                 "p99_spread": max(p99) / min(p99) if min(p99) > 0 else None},
            "bit_exact": mismatches == 0 and plain_bad == 0, "results_checked": checked + len(plain),
            "mismatches": mismatches + plain_bad,
            "plain_one_at_a_time": {"graphs_per_s": len(reqs) / plain_s, "seconds": plain_s,
                                    "speedup_of_served": statistics.median(gps) / (len(reqs) / plain_s)},
            "peak_device_bytes": st["peak_in_use"], "blocks": st["blocks"], "direct": st["direct"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--config", type=int, default=3, choices=[1, 2, 3, 4, 5])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-sub", action="store_true", help="skip the other single-graph workloads' sub-records")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched leg of the default run")
    ap.add_argument("--no-serve", action="store_true", help="skip the served leg of the default run")
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
            sv = served_leg(SERVED_REQUESTS, None, True, rates=SERVED_RATES)
        barrier()
        if rank == 0:
            sat = sv["saturated_passes"]
            line = {"metric": METRIC, "value": world * sv["saturated_graphs_per_s"], "unit": "graphs/s",
                    "n_gpus": world, "steps": sv["requests"], "warmup": 1,
                    "ms_per_step": 1e3 / sv["saturated_graphs_per_s"],
                    "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
                    "data": "synthetic", "config": graphs_config(5),
                    "p50_ms": statistics.median(sat["p50_ms"]), "p99_ms": statistics.median(sat["p99_ms"]),
                    "bit_exact": sv["bit_exact"],
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
                    "data": "synthetic", "config": graphs_config(4),
                    "roofline": {"bound": "hbm", "achieved": bl["hbm_gbs"], "peak": measured_peak_hbm()[0],
                                 "unit": "GB/s", "frac": bl["roofline_frac"], "traffic": None,
                                 "algorithmic_bytes": bl["algorithmic_bytes"]},
                    "gpu_launches": args.steps, "clocks": clk.summary(), "batched": bl}
            if "cpu_baseline" in bl:
                line["cpu_baseline"] = bl["cpu_baseline"]
            print(json.dumps(line), flush=True)
        return

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    if args.profile_e2e:
        off, nbr = W.single_graph(args.config)
        want, _ = O.bz(off, nbr)
        e2e_ms = e2e_leg(args, kc, len(off) - 1, len(nbr), off, nbr, want, flush, torch) * 1e3
        if rank == 0:
            print(json.dumps({"profile_run": True, "e2e_ms": e2e_ms, "workload": W.SINGLE[args.config]["name"]}),
                  flush=True)
        return

    head = single_leg(args.config, args, torch, flush, local, world, args.steps, args.warmup, full=True)
    if args.profile:
        if rank == 0:
            print(json.dumps({"profile_run": True, "ms_per_step": head["ms_per_step"],
                              "kernel_ms": head["kernel_ms"], "workload": head["workload"]}), flush=True)
        return
    if rank != 0 and world > 1:
        return
    line = {
        "metric": METRIC, "value": head["edges_per_s"], "unit": "edges/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": head["config"], "parallelism": f"replicas{world}",
        "hbm_gbs": head["hbm_gbs"], "arcs_per_s": head["arcs_per_s"], "kernel_ms": head["kernel_ms"],
        "roofline": head["roofline"], "e2e": head["e2e"], "gpu_launches": head["gpu_launches"],
        "method": head.get("method"), "iterations": head.get("iterations"),
        "clocks": head["clocks"], "wall_s": head["wall_s"], "bit_exact_vs_oracle": True,
    }
    for k in ("cpu_baseline", "reference_gpu"):
        if k in head:
            line[k] = head[k]
    if world == 1 and not args.no_sub:
        subs = {}
        for cfg in (1, 2, 3):
            if cfg == args.config:
                continue
            try:
                r = single_leg(cfg, args, torch, flush, local, world, max(3, args.steps // 2), max(3, args.warmup),
                               full=True)
                r.pop("config", None)
                subs[W.SINGLE[cfg]["name"]] = r
            except SystemExit as e:
                subs[W.SINGLE[cfg]["name"]] = {"error": str(e)}
        line["single_graph_workloads"] = subs
    if world == 1 and not args.no_batch:
        try:
            line["batched"] = batched_leg(argparse.Namespace(steps=5, warmup=3), torch, flush,
                                          with_cpu=not args.no_cpu)
        except Exception as e:   # the single-graph line stands on its own
            line["batched"] = {"error": repr(e)[:200]}
    if world == 1 and not args.no_serve:
        del flush
        torch.cuda.empty_cache()
        try:
            line["served"] = served_leg(SERVED_REQUESTS, None, True, rates=SERVED_RATES)
        except Exception as e:
            line["served"] = {"error": repr(e)[:200]}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
