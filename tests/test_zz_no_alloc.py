"""The allocation-free peel, kc_peel_noalloc, through the C ABI.

It exists for callers that cannot call cudaMalloc (a plugin host that owns all
device memory through its own pool, a latency-critical loop that must not pay
for allocation and the device-wide synchronisation it brings).  The test plays
such a caller: it owns the device buffers (allocated here with torch), hands
them to the entry point, and checks the core numbers and kmax of two calls in
a row, on two different graphs, bit for bit against the allocating entry point
kc_peel_csr and against the CPU oracle (Batagelj-Zaversnik).  The second call
also shows that the shared scratch is reset between calls; a run of 260 calls
alternating two graphs crosses the 8-bit wrap of the task-tag epoch, after
which stale queue entries must have been cleared.  This file sorts last so that
a run stopping at its first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import kcoregpu_gb300 as kc
from kcoregpu_gb300 import _lib
from oracle import kc_oracle as O

pytestmark = pytest.mark.gpu


def _noalloc_peel(torch, off, nbr, shift: int = 0):
    """shift > 0 places the CSR that many 4-byte words into its device buffers
    (pointers the caller owns need only 4-byte alignment)."""
    lib = kc.lib()
    V = len(off) - 1
    pad = np.zeros(shift, np.int32)
    d_off = torch.from_numpy(np.concatenate([pad, off.view(np.int32)])).cuda()
    d_nbr = torch.from_numpy(np.concatenate([pad, nbr.view(np.int32)])).cuda()
    d_core = torch.full((max(V, 1),), -1, dtype=torch.int32, device="cuda")
    kmax = C.c_uint32(12345)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.kc_peel_noalloc(C.c_void_p(d_off.data_ptr() + 4 * shift), C.c_void_p(d_nbr.data_ptr() + 4 * shift), V,
                             len(nbr), C.c_void_p(d_core.data_ptr()), C.byref(kmax), C.c_void_p(stream))
    _lib.check(rc, "kc_peel_noalloc")
    return d_core[:V].cpu().numpy().view(np.uint32), kmax.value


def test_noalloc_matches_allocating_entry_point_on_two_calls(gpu):
    torch = pytest.importorskip("torch")
    graphs = [kc.build_csr(*kc.gen_rmat(300_000, 2_000_000, seed=21))[:2],
              kc.build_csr(*kc.gen_chung_lu(400_000, 1_500_000, 2.1, 20_000.0, seed=22))[:2]]
    for off, nbr in graphs:   # two calls in a row on the shared scratch
        assert len(off) - 1 <= 524288 and len(nbr) <= 8388608   # KC_NOALLOC_MAX_V / _ARCS
        want, wk = kc.peel_csr(off, nbr)
        got, gk = _noalloc_peel(torch, off, nbr)
        np.testing.assert_array_equal(got, want)
        assert gk == wk
        bz, bk = O.bz(off, nbr)
        np.testing.assert_array_equal(got, bz)
        assert gk == bk


def test_noalloc_across_the_task_tag_wrap(gpu):
    # 260 calls alternating two graphs with hubs (queued tasks every call): the
    # calls just after the 255th reuse the queue with the tag epoch wrapped.
    torch = pytest.importorskip("torch")
    graphs = [kc.build_csr(*kc.gen_chung_lu(8_000, 40_000, 2.1, 2_000.0, seed=31))[:2],
              kc.build_csr(*kc.gen_rmat(6_000, 50_000, seed=32))[:2]]
    wants = [O.bz(off, nbr) for off, nbr in graphs]
    for i in range(260):
        off, nbr = graphs[i % 2]
        got, gk = _noalloc_peel(torch, off, nbr)
        want, wk = wants[i % 2]
        assert gk == wk, f"call {i}"
        np.testing.assert_array_equal(got, want, err_msg=f"call {i}")


def test_noalloc_rejects_graphs_beyond_its_limit(gpu):
    lib = kc.lib()
    kmax = C.c_uint32()
    rc = lib.kc_peel_noalloc(None, None, 524288 + 1, 0, None, C.byref(kmax), None)
    assert _lib.ERRORS[rc] == "KC_ERR_INVALID"
    assert b"scratch limits" in lib.kc_last_error()


def test_noalloc_refuses_an_invalid_csr_before_peeling(gpu):
    # The caller's device CSR is checked on the device before the peel
    # indexes with it: a neighbour id >= V and decreasing offsets are refused
    # with KC_ERR_INVALID, and the next valid call works.
    torch = pytest.importorskip("torch")
    off, nbr = kc.build_csr(*kc.gen_er(20_000, 80_000, seed=23))[:2]
    bad = nbr.copy()
    bad[len(bad) // 3] = len(off) - 1 + 1
    with pytest.raises(kc.KCoreError) as e:
        _noalloc_peel(torch, off, bad)
    assert e.value.name == "KC_ERR_INVALID"
    dec = off.copy()
    dec[100] = dec[99] - 1
    with pytest.raises(kc.KCoreError) as e:
        _noalloc_peel(torch, dec, nbr)
    assert e.value.name == "KC_ERR_INVALID"
    want, wk = kc.peel_csr(off, nbr)
    got, gk = _noalloc_peel(torch, off, nbr)
    np.testing.assert_array_equal(got, want)
    assert gk == wk


def test_noalloc_accepts_csr_arrays_at_4_byte_alignment(gpu):
    # Offsets and neighbour ids that start one word into their buffers: the
    # device-side CSR check then reads them with 4-byte loads instead of
    # 16-byte ones, and both the check and the peel give the same results.
    torch = pytest.importorskip("torch")
    off, nbr = kc.build_csr(*kc.gen_rmat(200_000, 1_500_000, seed=24))[:2]
    want, wk = kc.peel_csr(off, nbr)
    for shift in (1, 2, 3):
        got, gk = _noalloc_peel(torch, off, nbr, shift)
        np.testing.assert_array_equal(got, want)
        assert gk == wk
    bad = nbr.copy()
    bad[-5] = len(off) - 1
    with pytest.raises(kc.KCoreError) as e:
        _noalloc_peel(torch, off, bad, 1)
    assert e.value.name == "KC_ERR_INVALID"
