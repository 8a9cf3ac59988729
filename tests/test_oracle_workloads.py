"""The oracle's own workload generators (oracle/kc_gen_oracle.c) against the
product's: bench.py's reference arm builds its input graphs with the oracle's,
so both must give the same CSR bytes for every benchmark workload.

The single-graph workloads are compared at full size.  The batch and the
served stream are compared on their first graphs and requests.  The R-MAT
scale-24 graph is compared on the same generator at scale 18.  CPU only.
"""
import numpy as np
import pytest

from kcoregpu_gb300 import workloads as W
from oracle import kc_oracle as O
from oracle import kc_workloads as OW


def _same(a, b):
    return len(a) == len(b) and all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("cfg", [1, 2, 3])
def test_single_graph_workloads_identical(cfg):
    assert _same(W.single_graph(cfg), OW.single_graph(cfg))


def test_batch_workload_identical():
    a = W.batch(48)
    b = OW.batch(48)
    for k in ("vbase", "abase", "offsets", "neighbors"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    for g in (0, 1, 47):
        assert _same(OW.batch(48).graph(g), b.graph(g))


@pytest.mark.parametrize("i", range(8))
def test_served_requests_identical(i):
    assert _same(W.served_request(i, mmax=1_000_000), OW.served_request(i, mmax=1_000_000))


def test_served_big_generator_identical_small_scale():
    p = dict(W.served_big_params())
    p["n"], p["m"] = 1 << 18, (1 << 18) * 16
    import kcoregpu_gb300 as kc
    s, t = kc.gen_rmat(p["n"], p["m"], p["seed"])
    a = kc.build_csr(s, t)[:2]
    s2, t2 = O.gen_rmat(p["n"], p["m"], p["seed"])
    assert np.array_equal(s, s2) and np.array_equal(t, t2)
    assert _same(a, O.build_csr(s2, t2))


def test_er_and_csr_edge_cases():
    import kcoregpu_gb300 as kc
    for n, m, seed in [(2, 1, 3), (5, 10, 4), (1000, 20000, 5)]:
        assert _same(kc.gen_er(n, m, seed), O.gen_er(n, m, seed))
    # self-loops, duplicates and both directions collapse to one arc pair
    s = np.array([0, 1, 1, 2, 3, 3], np.uint32)
    t = np.array([1, 0, 1, 2, 0, 0], np.uint32)
    assert _same(kc.build_csr(s, t)[:2], O.build_csr(s, t))
