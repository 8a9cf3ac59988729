"""GPU parity of the batched peel: every graph of a batch bit-exact against the
oracle (per-graph Batagelj-Zaversnik), through the C ABI, including the
autotuner's grid-wide route for oversized graphs and the one-graph-per-launch
baseline."""
import numpy as np
import pytest

import kcoregpu_gb300 as kc
from kcoregpu_gb300 import batch as B
from oracle import kc_oracle as O

pytestmark = pytest.mark.gpu


def oracle(seg):
    return O.batch_bz(seg.vbase, seg.abase, seg.offsets, seg.neighbors, O.num_threads())


def test_generated_batch_matches_oracle(gpu):
    seg = B.gen_batch(96, 1000, nmin=1000, nmax=30000)
    want, wk = oracle(seg)
    b = B.Batch(seg)
    for _ in range(3):   # repeated passes over the same resident batch
        core, kmax, st = b.peel()
        np.testing.assert_array_equal(core, want)
        np.testing.assert_array_equal(kmax, wk)
    assert st["ngraphs"] == 96 and st["giants"] == 0
    plan = b.plan()
    assert sorted(plan["schedule"].tolist()) == list(range(96))
    b.free()


def test_edge_case_graphs_in_one_batch(gpu):
    graphs = []
    graphs.append(kc.build_csr([], []))                                   # V = 1, no arcs
    graphs.append(kc.build_csr([0], [0]))                                 # only a self-loop
    graphs.append(kc.build_csr(np.zeros(5000), np.arange(1, 5001)))       # star
    i, j = np.triu_indices(120, 1)
    graphs.append(kc.build_csr(i, j))                                     # K120
    graphs.append(kc.build_csr(np.arange(20000), np.arange(1, 20001)))    # long path
    graphs.append(kc.build_csr([3, 900], [900, 3]))                       # isolated ids
    graphs += [kc.build_csr(*kc.gen_chung_lu(3000 + 500 * k, 9000, 2.1, 400.0, 50 + k)) for k in range(6)]
    seg = B.Segmented.from_graphs([(o, n) for o, n, _ in graphs])
    want, wk = oracle(seg)
    core, kmax, st = B.Batch(seg).peel()
    np.testing.assert_array_equal(core, want)
    np.testing.assert_array_equal(kmax, wk)


def test_oversized_graph_goes_grid_wide(gpu):
    big = kc.build_csr(*kc.gen_rmat(300_000, 3_000_000, seed=77))
    small = [kc.build_csr(*kc.gen_er(2000, 8000, seed=80 + k)) for k in range(8)]
    seg = B.Segmented.from_graphs([(o, n) for o, n, _ in [small[0], big] + small[1:]])
    want, wk = oracle(seg)
    b = B.Batch(seg)
    core, kmax, st = b.peel()
    assert st["giants"] == 1 and b.plan()["schedule"][0] == 1
    np.testing.assert_array_equal(core, want)
    np.testing.assert_array_equal(kmax, wk)
    b.free()


def test_per_graph_baseline_agrees(gpu):
    seg = B.gen_batch(40, 7000, nmin=1000, nmax=20000)
    want, wk = oracle(seg)
    b = B.Batch(seg)
    ms = b.peel_per_graph()
    core, kmax, _ = b.fetch()
    np.testing.assert_array_equal(core, want)
    np.testing.assert_array_equal(kmax, wk)
    assert ms > 0
    b.free()
