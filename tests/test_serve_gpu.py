"""GPU tests of the served peel (continuous batching): every result bit-exact
against the oracle, and the same alone and in the mix; admission against the
HBM budget; a stream of many small requests."""
import numpy as np
import pytest

import kcoregpu_gb300 as kc
from kcoregpu_gb300 import KCoreError
from kcoregpu_gb300.serve import Server
from oracle import kc_oracle as O

pytestmark = pytest.mark.gpu


def mix():
    gs = []
    for k in range(6):   # small: one CTA each
        gs.append(kc.build_csr(*kc.gen_er(3000 + 700 * k, 12000 + 3000 * k, 300 + k))[:2])
    gs.append(kc.build_csr(*kc.gen_rmat(250_000, 2_500_000, 310))[:2])          # gang of 2
    gs.append(kc.build_csr(*kc.gen_chung_lu(600_000, 2_000_000, 2.1, 20_000.0, 311))[:2])  # large V
    gs.append(kc.build_csr(*kc.gen_rmat(1 << 20, 6 << 20, 312))[:2])             # gang of ~5
    i, j = np.triu_indices(300, 1)
    gs.append(kc.build_csr(i, j)[:2])
    gs.append(kc.build_csr(np.arange(50_000), np.arange(1, 50_001))[:2])         # long path
    return gs


def test_each_result_same_alone_and_in_the_mix(gpu):
    gs = mix()
    want = [O.bz(o, n) for o, n in gs]
    srv = Server()
    alone = []
    for o, n in gs:
        core, kmax, t = srv.wait(srv.submit(o, n))
        alone.append((core, kmax, t))
    ids = [srv.submit(o, n) for o, n in gs]          # all in flight together
    together = [srv.wait(r) for r in ids]
    srv.close()
    for (wc, wk), (ac, ak, at), (tc, tk, tt) in zip(want, alone, together):
        np.testing.assert_array_equal(ac, wc)
        np.testing.assert_array_equal(tc, wc)
        assert ak == wk == tk
    assert max(t["gang"] for _, _, t in together) > 1     # some ran as gangs


def test_admission_against_a_small_budget(gpu):
    gs = mix()[:8]
    need = max(4 * (len(o) + len(n)) for o, n in gs)
    srv = Server(hbm_budget_bytes=int(need * 3.5))
    ids = [srv.submit(o, n) for o, n in gs]
    res = [srv.wait(r) for r in ids]
    st = srv.stats()
    assert st["peak_in_use"] <= need * 3.5 and st["completed"] == len(gs)
    for (o, n), (core, kmax, _) in zip(gs, res):
        wc, wk = O.bz(o, n)
        np.testing.assert_array_equal(core, wc)
        assert kmax == wk
    big = kc.build_csr(*kc.gen_rmat(1 << 20, 8 << 20, 5))[:2]
    with pytest.raises(KCoreError) as e:
        srv.submit(*big)
    assert e.value.name == "KC_ERR_BUDGET"
    srv.close()


def test_stream_of_small_requests(gpu):
    gs = [kc.build_csr(*kc.gen_rmat(2000 + 37 * k, 9000 + 91 * k, 900 + k))[:2] for k in range(200)]
    srv = Server()
    ids = [srv.submit(o, n) for o, n in gs]
    for (o, n), r in zip(gs, ids):
        core, kmax, _ = srv.wait(r)
        wc, wk = O.bz(o, n)
        np.testing.assert_array_equal(core, wc)
        assert kmax == wk
    srv.close()


@pytest.mark.parametrize("staged", ["0", "1"])
def test_direct_and_staged_transfers_agree(gpu, monkeypatch, staged):
    # On devices that reach pageable host memory the gangs copy each request's
    # CSR in and its result out themselves; KC_SERVE_STAGED=1 forces the pinned
    # staging path.  Both must give the oracle's results, for arrays with and
    # without 16-byte alignment.
    monkeypatch.setenv("KC_SERVE_STAGED", staged)
    gs = mix()[:9]
    o, n = gs[6]
    buf = np.empty(len(n) + 1, np.uint32)     # neighbours at a 4-byte (not 16-byte) offset
    buf[1:] = n
    gs.append((o, buf[1:]))
    srv = Server()
    direct = srv.stats()["direct"]
    if staged == "1":
        assert direct == 0
    ids = [srv.submit(o, n) for o, n in gs]
    res = [srv.wait(r) for r in ids]
    srv.close()
    for (o, n), (core, kmax, _) in zip(gs, res):
        wc, wk = O.bz(o, n)
        np.testing.assert_array_equal(core, wc)
        assert kmax == wk


@pytest.mark.parametrize("staged", ["0", "1"])
def test_malformed_requests_are_refused_and_the_server_continues(gpu, monkeypatch, staged):
    # A neighbour id >= V is refused before any kernel indexes with it: on the
    # host with pinned staging, while the gang copies the CSR in otherwise (for
    # a one-CTA job and for a gang).  Decreasing offsets fail the submit.
    monkeypatch.setenv("KC_SERVE_STAGED", staged)
    srv = Server()
    small = kc.build_csr(*kc.gen_er(5000, 20000, 77))[:2]
    big = kc.build_csr(*kc.gen_rmat(1 << 20, 6 << 20, 78))[:2]
    for o, n in (small, big):
        bad = n.copy()
        bad[len(bad) // 2] = len(o) - 1 + 5     # >= V
        if staged == "1":
            with pytest.raises(KCoreError) as e:
                srv.submit(o, bad)
        else:
            rid = srv.submit(o, bad)
            with pytest.raises(KCoreError) as e:
                srv.wait(rid)
        assert e.value.name == "KC_ERR_INVALID"
    o, n = small
    dec = o.copy()
    dec[11] = dec[10] - 1                    # offsets decrease
    with pytest.raises(KCoreError) as e:
        srv.submit(dec, n)
    assert e.value.name == "KC_ERR_INVALID"
    for o, n in (small, big):    # the server still serves
        core, kmax, t = srv.wait(srv.submit(o, n))
        wc, wk = O.bz(o, n)
        np.testing.assert_array_equal(core, wc)
        assert kmax == wk
        assert t["peel_us"] > 0
    srv.close()


@pytest.mark.slow
def test_served_config_with_the_scale24_graph(gpu):
    """The served workload's R-MAT scale-24 edge-factor-16 graph (2^24
    vertices, 2^28 draws, ~407 M undirected edges), bit for bit against BZ:
    through the server alone, inside a mix of the stream's first requests,
    and through the one-shot kc_peel_csr."""
    from kcoregpu_gb300 import workloads as W
    big = W.served_big()
    reqs = [W.served_request(i, mmax=2_000_000) for i in range(6)]
    want_big = O.bz(*big)
    wants = [O.bz(*r) for r in reqs]
    srv = Server()
    core, kmax, t = srv.wait(srv.submit(*big), timeout_s=300)
    np.testing.assert_array_equal(core, want_big[0])
    assert kmax == want_big[1]
    ids = [srv.submit(*r) for r in reqs[:3]] + [srv.submit(*big)] + [srv.submit(*r) for r in reqs[3:]]
    res = [srv.wait(r, timeout_s=300) for r in ids]
    srv.close()
    order = wants[:3] + [want_big] + wants[3:]
    for (c, k, _), (wc, wk) in zip(res, order):
        np.testing.assert_array_equal(c, wc)
        assert k == wk
    core, kmax = kc.peel_csr(*big)
    np.testing.assert_array_equal(core, want_big[0])
    assert kmax == want_big[1]
