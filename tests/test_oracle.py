"""The oracle pinned against the golden vectors (CPU only).

Both oracle restatements (the reference's level-synchronous peel and the
Batagelj-Zaversnik bucket peel) must reproduce networkx.core_number on the
reference loader's own CSR for every fixture before any GPU result is judged
against them.
"""
import numpy as np
import pytest

from conftest import golden_core, golden_names, golden_serialized
from oracle import kc_oracle as O


@pytest.mark.parametrize("name", golden_names(include_quirks=True))
def test_bz_matches_networkx(name):
    off, nbr, _ = golden_serialized(name)
    core, kmax = O.bz(off, nbr)
    want = golden_core(name)
    np.testing.assert_array_equal(core, want)
    assert kmax == int(want.max())


@pytest.mark.parametrize("name", golden_names(include_quirks=True))
@pytest.mark.parametrize("threads", [1, 4])
def test_levelsync_matches_networkx(name, threads):
    off, nbr, _ = golden_serialized(name)
    core, kmax, levels, order, shells = O.levelsync(off, nbr, nthreads=threads, with_order=True)
    want = golden_core(name)
    np.testing.assert_array_equal(core, want)
    assert kmax == int(want.max())
    assert levels == kmax + 1
    # peel order is a permutation and the k-shell offsets delimit it by level
    V = len(off) - 1
    assert sorted(order.tolist()) == list(range(V))
    assert shells[0] == 0 and shells[-1] == V
    for k in range(kmax + 1):
        assert (core[order[shells[k]:shells[k + 1]]] == k).all()


def test_empty_graph_kmax_wraps_like_reference():
    # ours.cc:151 sets kmax = level-1 with level == 0 when the loop never runs
    off = np.zeros(1, np.uint32)
    nbr = np.zeros(0, np.uint32)
    assert O.bz(off, nbr)[1] == 0xFFFFFFFF
    assert O.levelsync(off, nbr)[1] == 0xFFFFFFFF


def test_oracles_agree_on_random_graphs():
    rng = np.random.default_rng(7)
    import kcoregpu_gb300 as kc
    for trial in range(5):
        n = int(rng.integers(50, 5000))
        m = int(rng.integers(n, 8 * n))
        off, nbr, _ = kc.build_csr(rng.integers(0, n, m), rng.integers(0, n, m))
        a, ka = O.bz(off, nbr)
        b, kb, _ = O.levelsync(off, nbr, nthreads=8)
        np.testing.assert_array_equal(a, b)
        assert ka == kb


def test_parity_comparison_detects_a_planted_error():
    # A planted mistake lives in the oracle's output, on the CPU: the parity
    # comparison used by the GPU tests must reject it.
    off, nbr, _ = golden_serialized("two_cliques")
    core, _ = O.bz(off, nbr)
    bad = core.copy()
    bad[3] += 1
    with pytest.raises(AssertionError):
        np.testing.assert_array_equal(bad, golden_core("two_cliques"))


def test_batch_bz_matches_per_graph():
    import kcoregpu_gb300 as kc
    rng = np.random.default_rng(3)
    offs, nbrs, cores, vb, ab = [], [], [], [0], [0]
    for g in range(6):
        n = int(rng.integers(20, 400))
        off, nbr, _ = kc.build_csr(rng.integers(0, n, 3 * n), rng.integers(0, n, 3 * n))
        c, _ = O.bz(off, nbr)
        offs.append(off); nbrs.append(nbr); cores.append(c)
        vb.append(vb[-1] + len(off) - 1); ab.append(ab[-1] + len(nbr))
    core, kmax = O.batch_bz(np.array(vb, np.uint64), np.array(ab, np.uint64),
                            np.concatenate(offs), np.concatenate(nbrs), 4)
    np.testing.assert_array_equal(core, np.concatenate(cores))
    assert list(kmax) == [int(c.max()) for c in cores]
