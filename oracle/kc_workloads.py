"""TEST INFRASTRUCTURE ONLY: the benchmark workloads built by the oracle's own
generators and CSR builder (kc_gen_oracle.c) instead of the product library.

bench.py's reference arm takes its input graphs from here, so that arm maps
no product library; tests/test_oracle_workloads.py requires every CSR made here
to equal, byte for byte, the one kcoregpu_gb300.workloads makes.  The
workload parameters (sizes, seeds) come from kcoregpu_gb300.workloads, a pure
Python module that loads nothing until one of its generators is called.
"""
from __future__ import annotations

import functools

import numpy as np

from kcoregpu_gb300 import workloads as W

from . import kc_oracle as O


def _graph(p: dict):
    if p["kind"] == "rmat":
        s, t = O.gen_rmat(p["n"], p["m"], p["seed"])
    elif p["kind"] == "chung_lu":
        s, t = O.gen_chung_lu(p["n"], p["m"], p["gamma"], p["max_w"], p["seed"])
    else:
        s, t = O.gen_er(p["n"], p["m"], p["seed"])
    return O.build_csr(s, t)


@functools.lru_cache(maxsize=3)
def single_graph(cfg: int):
    """-> (offsets, neighbors) of single-graph workload `cfg` (1, 2 or 3)."""
    c = W.SINGLE[cfg]
    if c["kind"] == "rmat":
        return _graph(dict(kind="rmat", n=c["n"], m=c["edges"], seed=c["seed"]))
    return _graph(dict(kind="chung_lu", n=c["n"], m=c["edges"], gamma=c["gamma"], max_w=c["max_w"], seed=c["seed"]))


class Segmented:
    """A segmented CSR (graph g: vbase/abase bases, V_g+1 local offsets at
    vbase[g]+g, local neighbour ids at abase[g])."""

    def __init__(self, vbase, abase, offsets, neighbors):
        self.vbase, self.abase, self.offsets, self.neighbors = vbase, abase, offsets, neighbors

    @property
    def ngraphs(self) -> int:
        return len(self.vbase) - 1

    def graph(self, g: int):
        v0, v1 = int(self.vbase[g]), int(self.vbase[g + 1])
        a0, a1 = int(self.abase[g]), int(self.abase[g + 1])
        return self.offsets[v0 + g: v1 + g + 1], self.neighbors[a0:a1]


def batch(ngraphs: int | None = None) -> Segmented:
    """The batched workload (first `ngraphs` graphs of it)."""
    c = W.BATCH
    return Segmented(*O.gen_batch(ngraphs or c["ngraphs"], c["seed_base"], c["nmin"], c["nmax"], c["dmin"],
                                  c["dmax"]))


def served_request(i: int, mmin: int | None = None, mmax: int | None = None):
    """Request i of the served stream -> (offsets, neighbors)."""
    return _graph(W.served_params(i, mmin, mmax))


def served_big():
    """The R-MAT scale-24 edge-factor-16 graph of the served stream."""
    return _graph(W.served_big_params())


def equal_csr(a, b) -> bool:
    return all(np.array_equal(x, y) for x, y in zip(a, b))
