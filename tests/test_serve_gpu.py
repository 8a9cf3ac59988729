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
