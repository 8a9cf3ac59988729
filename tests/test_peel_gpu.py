"""GPU parity of the persistent peel, through the C ABI: bit-exact uint32 core
numbers and kmax against the oracle (networkx-pinned) on the golden fixtures,
adversarial shapes, and the three single-graph workloads at full size."""
import numpy as np
import pytest

import kcoregpu_gb300 as kc
from conftest import golden_core, golden_names, golden_serialized
from kcoregpu_gb300 import KCoreError
from oracle import kc_oracle as O

pytestmark = pytest.mark.gpu


def check(off, nbr, core, kmax):
    want, wk = O.bz(off, nbr)
    np.testing.assert_array_equal(core, want)
    assert kmax == wk


@pytest.mark.parametrize("name", golden_names(include_quirks=True))
def test_golden_fixtures(gpu, name):
    off, nbr, _ = golden_serialized(name)
    core, kmax = kc.peel_csr(off, nbr)
    want = golden_core(name)
    np.testing.assert_array_equal(core, want)
    assert kmax == int(want.max())


def test_empty_graph_kmax(gpu):
    core, kmax = kc.peel_csr(np.zeros(1, np.uint32), np.zeros(0, np.uint32))
    assert len(core) == 0 and kmax == 0xFFFFFFFF   # ours.cc:151 with level == 0


@pytest.mark.parametrize("shape", ["star", "clique", "path", "isolated", "hub_of_leaves",
                                   "two_hubs", "ladder"])
def test_adversarial_shapes(gpu, shape):
    if shape == "star":
        s, t = np.zeros(200000, np.uint32), np.arange(1, 200001, dtype=np.uint32)
    elif shape == "clique":
        i, j = np.triu_indices(400, 1)
        s, t = i.astype(np.uint32), j.astype(np.uint32)
    elif shape == "path":   # one long cascade inside level 1
        s = np.arange(0, 300000, dtype=np.uint32)
        t = s + 1
    elif shape == "isolated":
        s, t = np.array([5, 1000000], np.uint32), np.array([7, 999999], np.uint32)
    elif shape == "hub_of_leaves":   # hub with many degree-1 leaves and a clique core
        i, j = np.triu_indices(60, 1)
        s = np.concatenate([i, np.zeros(100000)]).astype(np.uint32)
        t = np.concatenate([j, np.arange(60, 100060)]).astype(np.uint32)
    elif shape == "two_hubs":
        leaves = np.arange(2, 150002, dtype=np.uint32)
        s = np.concatenate([np.zeros(len(leaves), np.uint32), np.ones(len(leaves), np.uint32)])
        t = np.concatenate([leaves, leaves])
    else:   # ladder: many equal-degree vertices, deep cascades
        n = 100000
        a = np.arange(n - 1, dtype=np.uint32)
        s = np.concatenate([a, a + n, np.arange(n, dtype=np.uint32)])
        t = np.concatenate([a + 1, a + n + 1, np.arange(n, dtype=np.uint32) + n])
    off, nbr, _ = kc.build_csr(s, t)
    core, kmax = kc.peel_csr(off, nbr)
    check(off, nbr, core, kmax)


@pytest.mark.parametrize("seed", range(6))
def test_random_graphs(gpu, seed):
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(1000, 200000))
    m = int(n * rng.uniform(2, 30))
    if seed % 3 == 0:
        s, t = kc.gen_er(n, m, seed)
    elif seed % 3 == 1:
        s, t = kc.gen_rmat(n, m, seed)
    else:
        s, t = kc.gen_chung_lu(n, m // 2, 2.1 + 0.1 * seed, n / 20.0, seed)
    off, nbr, _ = kc.build_csr(s, t)
    core, kmax = kc.peel_csr(off, nbr)
    check(off, nbr, core, kmax)


def test_device_graph_repeated_peels_and_epoch_wrap(gpu):
    s, t = kc.gen_rmat(20000, 120000, seed=4)
    off, nbr, _ = kc.build_csr(s, t)
    want, wk = O.bz(off, nbr)
    g = kc.DeviceGraph(off, nbr)
    for i in range(300):   # task tags wrap after 255 runs
        core, kmax, st = g.peel()
        if i % 50 == 0 or i > 250:
            np.testing.assert_array_equal(core, want)
            assert kmax == wk and st["levels"] == wk + 1
    g.free()


def test_degeneracy_order_and_shells(gpu):
    s, t = kc.gen_chung_lu(50000, 150000, 2.2, 3000.0, seed=8)
    off, nbr, _ = kc.build_csr(s, t)
    g = kc.DeviceGraph(off, nbr)
    order, shells, kmax = g.degeneracy_order()
    core, wk = O.bz(off, nbr)
    V = len(off) - 1
    assert kmax == wk
    assert np.array_equal(np.sort(order), np.arange(V, dtype=np.uint32))
    assert shells[0] == 0 and shells[-1] == V and len(shells) == kmax + 2
    for k in range(kmax + 1):
        assert (core[order[shells[k]:shells[k + 1]]] == k).all()
    # the order is a valid degeneracy order: when v is removed, at most
    # core(v) of its neighbours come later
    pos = np.empty(V, np.int64)
    pos[order] = np.arange(V)
    src = np.repeat(np.arange(V), np.diff(off))
    later = np.bincount(src[pos[nbr] > pos[src]], minlength=V)
    assert (later <= core).all()
    g.free()


@pytest.mark.slow
@pytest.mark.parametrize("cfg", [1, 2, 3])
def test_full_size_workloads(gpu, cfg):
    from kcoregpu_gb300 import workloads
    off, nbr = workloads.single_graph(cfg)
    core, kmax = kc.peel_csr(off, nbr)
    check(off, nbr, core, kmax)
    # size-independent properties on top of the oracle: every vertex of core k
    # keeps >= k neighbours of core >= k (k-core definition), and core <= degree
    deg = np.diff(off)
    assert (core <= deg).all()
    src = np.repeat(np.arange(len(deg)), deg)
    strong = np.bincount(src[core[nbr] >= core[src]], minlength=len(deg))
    assert (strong >= core).all()


@pytest.mark.slow
@pytest.mark.parametrize("cfg", [2, 3])
def test_repeated_full_size_peels_are_stable(gpu, cfg):
    # Every repetition must reproduce the oracle: a race in the level
    # completion protocol shows up here as a wrong core number.
    from kcoregpu_gb300 import workloads
    off, nbr = workloads.single_graph(cfg)
    want, wk = O.bz(off, nbr)
    g = kc.DeviceGraph(off, nbr)
    for _ in range(25):
        core, kmax, _ = g.peel()
        np.testing.assert_array_equal(core, want)
        assert kmax == wk
    tr = g.trace()
    assert 1 <= len(tr) <= wk + 1 and int(tr[-1, 4]) == len(off) - 1
    g.free()


def test_one_shot_peel_refuses_invalid_csr_on_the_device(gpu):
    # kc_peel_csr checks the CSR on the device after the upload: an invalid
    # graph is refused with KC_ERR_INVALID before the peel touches it, and the
    # next valid call is unaffected.  (kc_graph_upload still checks at upload.)
    off, nbr = kc.build_csr(*kc.gen_rmat(50_000, 300_000, seed=31))[:2]
    want, wk = O.bz(off, nbr)
    bad = nbr.copy()
    bad[-1] = len(off) - 1 + 3
    with pytest.raises(KCoreError) as e:
        kc.peel_csr(off, bad)
    assert e.value.name == "KC_ERR_INVALID"
    dec = off.copy()
    dec[500] = dec[499] - 1
    with pytest.raises(KCoreError) as e:
        kc.peel_csr(dec, nbr)
    assert e.value.name == "KC_ERR_INVALID"
    core, k = kc.peel_csr(off, nbr)
    np.testing.assert_array_equal(core, want)
    assert k == wk
    with pytest.raises(KCoreError) as e:
        kc.DeviceGraph(off, bad)
    assert e.value.name == "KC_ERR_INVALID"
