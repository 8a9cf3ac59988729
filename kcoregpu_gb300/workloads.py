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
