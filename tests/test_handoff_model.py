"""A model of the h-index peel's hand-off to the cluster kernel, checked on CPU.

The device iteration (kcoregpu_gb300/csrc/kc_hindex.cu) replaces each queued
vertex's estimate by the h-index of its neighbours' estimates; the queued
vertices of the next iteration are those whose estimate would fall.  Once the
frontier is small the grid hands the rest to the cluster kernel
(kcoregpu_gb300/csrc/kc_hxtail.cu): S = {v : est[v] >= T}, T the smallest of
T0/2, 5T0/8, ..., T0 (T0 the frontier's smallest estimate) that leaves at most
a given number of vertices in S, and only when every member of S has at least
T neighbours in S (counting repeated arcs, as the device does).  The model
runs the same rule with synchronous iterations (any order of updates reaches
the same fixed point, since every estimate stays an upper bound) and checks:
  * every queued vertex lies in S;
  * when the certificate holds, every vertex outside S already has its core
    number, and finishing S alone, with floor T, from the handed-over
    estimates gives the core numbers of the whole graph (the oracle's);
  * that holds at every iteration where the hand-off qualifies;
  * without the certificate the split can be wrong (a star: the hub alone
    would keep the floor as its core number).
Graphs: R-MAT, Chung-Lu and Erdos-Renyi from the oracle's generators, and a
raw CSR with repeated arcs and self-loops.
"""
import numpy as np
import pytest

from oracle import kc_oracle as O


def hindex_step(off, nbr, est, floor=0):
    """One synchronous h-index step: new[v] = max(floor, min(est[v], h-index of est[N(v)]))."""
    V = len(off) - 1
    new = est.copy()
    for v in range(V):
        xs = np.sort(est[nbr[off[v]:off[v + 1]]])[::-1]
        # largest h with at least h values >= h
        ks = np.arange(1, len(xs) + 1)
        ok = xs >= ks
        h = int(ks[ok][-1]) if ok.any() else 0
        new[v] = max(floor, min(est[v], h))
    return new


def cand_floor(t0, k):
    return max(1, (t0 * (4 + k)) // 8)


def try_handoff(off, nbr, est, nmax):
    """The device's choice of S; None when no floor fits or the certificate fails."""
    nxt = hindex_step(off, nbr, est)
    frontier = np.nonzero(nxt < est)[0]
    if len(frontier) == 0:
        return None
    t0 = int(est[frontier].min())
    if t0 < 2:
        return None
    for k in range(5):
        T = cand_floor(t0, k)
        inS = est >= T
        if 0 < inS.sum() <= nmax:
            break
    else:
        return None
    assert inS[frontier].all(), "a queued vertex lies outside S"
    deg_in = np.array([int(inS[nbr[off[v]:off[v + 1]]].sum()) for v in range(len(off) - 1)])
    if (deg_in[inS] < T).any():
        return None
    return T, inS


def finish_inside(off, nbr, est, T, inS):
    """The cluster's part: iterate on the induced subgraph of S with floor T."""
    ids = np.nonzero(inS)[0]
    lid = -np.ones(len(off) - 1, np.int64)
    lid[ids] = np.arange(len(ids))
    soff = [0]
    snbr = []
    for v in ids:
        ns = nbr[off[v]:off[v + 1]]
        ns = lid[ns[inS[ns]]]
        snbr.extend(ns.tolist())
        soff.append(len(snbr))
    soff = np.array(soff, np.int64)
    snbr = np.array(snbr, np.int64)
    e = est[ids].copy()
    for _ in range(10_000):
        n = hindex_step(soff, snbr, e, floor=T)
        if np.array_equal(n, e):
            break
        e = n
    out = est.copy()
    out[ids] = e
    return out


def run_model(off, nbr, nmax):
    off = np.asarray(off, np.int64)
    nbr = np.asarray(nbr, np.int64)
    want, _ = O.bz(off.astype(np.uint32), nbr.astype(np.uint32))
    want = want.astype(np.int64)
    est = np.diff(off)
    handed = 0
    for _ in range(10_000):
        ho = try_handoff(off, nbr, est, nmax)
        if ho is not None:
            T, inS = ho
            # outside S the estimates are already final
            np.testing.assert_array_equal(est[~inS], want[~inS])
            np.testing.assert_array_equal(finish_inside(off, nbr, est, T, inS), want)
            handed += 1
        nxt = hindex_step(off, nbr, est)
        if np.array_equal(nxt, est):
            break
        est = nxt
    np.testing.assert_array_equal(est, want)
    return handed


def _csr(s, t):
    off, nbr = O.build_csr(np.asarray(s, np.uint32), np.asarray(t, np.uint32))
    return off, nbr


GRAPHS = {
    "rmat-3k": lambda: _csr(*O.gen_rmat(3_000, 24_000, 7)),
    "chunglu-4k": lambda: _csr(*O.gen_chung_lu(4_000, 20_000, 2.1, 600.0, 8)),
    "er-2k": lambda: _csr(*O.gen_er(2_000, 10_000, 9)),
}


@pytest.mark.parametrize("name", sorted(GRAPHS))
@pytest.mark.parametrize("nmax", [64, 512, 1 << 20])
def test_handoff_gives_the_core_numbers(name, nmax):
    off, nbr = GRAPHS[name]()
    handed = run_model(off, nbr, nmax)
    if nmax == 1 << 20:
        assert handed > 0   # with no size limit some iteration qualifies


def test_handoff_with_repeated_arcs_and_self_loops():
    rng = np.random.default_rng(3)
    V = 400
    s0 = rng.integers(0, V, 3_000)
    t0 = rng.integers(0, V, 3_000)
    loops = np.arange(0, V, 5)
    s = np.concatenate([s0, t0, loops])
    t = np.concatenate([t0, s0, loops])
    order = np.lexsort((t, s))
    s, t = s[order], t[order]
    off = np.zeros(V + 1, np.int64)
    np.add.at(off, s + 1, 1)
    off = np.cumsum(off)
    # the reference rule (every arc counts; a self-loop never drops its vertex)
    # is what the level-synchronous oracle computes on a raw CSR
    want, _, _, _, _ = O.levelsync(off.astype(np.uint32), t.astype(np.uint32), nthreads=1, with_order=True)
    est = np.diff(off)
    nbr = t.astype(np.int64)
    for _ in range(10_000):
        ho = try_handoff(off, nbr, est, 1 << 20)
        if ho is not None:
            T, inS = ho
            np.testing.assert_array_equal(est[~inS], want[~inS].astype(np.int64))
            np.testing.assert_array_equal(finish_inside(off, nbr, est, T, inS), want.astype(np.int64))
        nxt = hindex_step(off, nbr, est)
        if np.array_equal(nxt, est):
            break
        est = nxt
    np.testing.assert_array_equal(est, want.astype(np.int64))


def test_certificate_refuses_a_star():
    # a hub of degree 20 among leaves: the frontier is the hub (estimate 20),
    # S = {hub} for every candidate floor, and the hub has no neighbour in S
    off, nbr = _csr(np.zeros(20), np.arange(1, 21))
    off = np.asarray(off, np.int64)
    nbr = np.asarray(nbr, np.int64)
    est = np.diff(off)
    assert try_handoff(off, nbr, est, 1 << 20) is None
    inS = est >= 10
    assert inS.sum() == 1
    wrong = finish_inside(off, nbr, est, 10, inS)
    want, _ = O.bz(off.astype(np.uint32), nbr.astype(np.uint32))
    assert wrong[0] == 10 and want[0] == 1   # what the certificate prevents
