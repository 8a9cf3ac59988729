"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference names three SNAP datasets (amazon0601, web-Google, wiki-Talk)
that are not available; these generators stand in for them with fixed seeds.
"""
from __future__ import annotations

import functools

import numpy as np

from . import graph as G

SINGLE = {
    1: dict(name="rmat-400k-3.4M", kind="rmat", n=400_000, edges=3_400_000, seed=1),
    2: dict(name="rmat-s20-ef5", kind="rmat", n=1 << 20, edges=5 << 20, seed=2),
    3: dict(name="chunglu-2.4M-g2.1", kind="chung_lu", n=2_400_000, edges=5_000_000, seed=3,
            gamma=2.1, max_w=100_000.0),
}


def edges(cfg: int):
    c = SINGLE[cfg]
    if c["kind"] == "rmat":
        return G.gen_rmat(c["n"], c["edges"], c["seed"])
    return G.gen_chung_lu(c["n"], c["edges"], c["gamma"], c["max_w"], c["seed"])


@functools.lru_cache(maxsize=3)
def single_graph(cfg: int):
    """-> (offsets, neighbors) of single-graph workload `cfg` (1, 2 or 3)."""
    s, t = edges(cfg)
    off, nbr, _ = G.build_csr(s, t)
    return off, nbr


def algorithmic_bytes(V: int, arcs: int, kmax: int) -> int:
    """Bytes of one level-synchronous peel: offsets once, each arc once per
    peeled endpoint, one degree-array pass per level (kmax+1 levels)."""
    return 4 * (V + 1) + 4 * arcs + 4 * V * (kmax + 1)


BATCH = dict(name="batch-4096-er-rmat", ngraphs=4096, seed_base=1000, nmin=1000, nmax=200_000,
             dmin=4.0, dmax=32.0)


def batch(ngraphs: int | None = None):
    """The batched workload: graph g uses seed 1000+g, n ~ log-uniform[1,000,
    200,000], average degree 2m/n ~ U[4,32], even g Erdos-Renyi, odd g R-MAT."""
    from .batch import gen_batch
    c = BATCH
    return gen_batch(ngraphs or c["ngraphs"], c["seed_base"], c["nmin"], c["nmax"], c["dmin"], c["dmax"])


def batch_algorithmic_bytes(seg, kmax) -> int:
    """Sum over the graphs of the single-graph formula."""
    import numpy as np
    V = np.diff(seg.vbase).astype(np.int64)
    A = np.diff(seg.abase).astype(np.int64)
    k = np.asarray(kmax, dtype=np.int64)
    k = np.where(k == 0xFFFFFFFF, -1, k)
    return int((4 * (V + 1) + 4 * A + 4 * V * (k + 1)).sum())


SERVED = dict(name="served-poisson-rmat-chunglu+rmat-s24", requests=240, seed_base=5000, mmin=10_000,
              mmax=8_000_000, big_position=120, big_scale=24, big_edge_factor=16)


def served_params(i: int, mmin: int | None = None, mmax: int | None = None) -> dict:
    """Generator parameters of request i of the served stream: m ~
    log-uniform[10K, 8M] undirected edges, alternating R-MAT (m draws, n = m/8
    vertices) and Chung-Lu (gamma ~ U[2.1, 2.5], n = m/4, max weight
    sqrt(n)*8), seed 5000+i."""
    import math
    import numpy as np
    c = SERVED
    lo, hi = mmin or c["mmin"], mmax or c["mmax"]
    rng = np.random.default_rng(c["seed_base"] + i)
    m = int(math.exp(rng.uniform(math.log(lo), math.log(hi))))
    seed = c["seed_base"] + i
    if i % 2 == 0:
        return dict(kind="rmat", n=max(64, m // 8), m=m, seed=seed)
    n = max(64, m // 4)
    return dict(kind="chung_lu", n=n, m=m, gamma=float(rng.uniform(2.1, 2.5)), max_w=math.sqrt(n) * 8.0, seed=seed)


def served_request(i: int, mmin: int | None = None, mmax: int | None = None):
    """Request i of the served stream (served_params) -> (offsets, neighbors)."""
    p = served_params(i, mmin, mmax)
    if p["kind"] == "rmat":
        s, t = G.gen_rmat(p["n"], p["m"], p["seed"])
    else:
        s, t = G.gen_chung_lu(p["n"], p["m"], p["gamma"], p["max_w"], p["seed"])
    off, nbr, _ = G.build_csr(s, t)
    return off, nbr


def served_big_params() -> dict:
    """The R-MAT scale-24 edge-factor-16 graph of the served stream."""
    c = SERVED
    n = 1 << c["big_scale"]
    return dict(kind="rmat", n=n, m=n * c["big_edge_factor"], seed=c["seed_base"] + 99999)


def served_big():
    """The R-MAT scale-24 edge-factor-16 graph (2^24 vertices, 2^28 draws)."""
    p = served_big_params()
    s, t = G.gen_rmat(p["n"], p["m"], p["seed"])
    off, nbr, _ = G.build_csr(s, t)
    return off, nbr
