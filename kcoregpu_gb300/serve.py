"""Served peel: continuous batching of k-core requests (C ABI kc_serve_*).
No reference counterpart: the reference peels one graph per process."""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import _lib as L
from ._lib import check, lib, ptr, u32


class Server:
    """A running server: submit CSR graphs, poll or wait for core numbers."""

    def __init__(self, hbm_budget_bytes: int = 0, ring_slots: int = 0, gang_arcs: int = 0,
                 max_gang: int = 0, small_vertices: int = 0):
        cfg = L.ServeCfg(hbm_budget_bytes, ring_slots, gang_arcs, max_gang, small_vertices)
        h = C.c_void_p()
        check(lib().kc_serve_open(C.byref(cfg), C.byref(h)), "kc_serve_open")
        self._h = h
        self._live = {}   # request id -> (offsets, neighbors, core): kept alive until done
        self._mu = threading.Lock()

    def submit(self, offsets, neighbors) -> int:
        off, nbr = u32(offsets), u32(neighbors)
        V = len(off) - 1
        core = np.empty(max(V, 1), np.uint32)
        rid = C.c_uint64()
        check(lib().kc_serve_submit(self._h, ptr(off), ptr(nbr) if len(nbr) else None, V, ptr(core),
                                    C.byref(rid)), "kc_serve_submit")
        with self._mu:
            self._live[rid.value] = (off, nbr, core, V)
        return rid.value

    def _finish(self, rid, rc, kmax, t):
        if rc == -10:   # KC_ERR_BUSY
            return None
        with self._mu:
            off, nbr, core, V = self._live.pop(rid)
        check(rc, "kc_serve_result")
        return core[:V], kmax.value, t.as_dict()

    def poll(self, rid: int):
        """-> (core, kmax, timing) when done, else None."""
        kmax, t = C.c_uint32(), L.ServeTiming()
        rc = lib().kc_serve_poll(self._h, rid, C.byref(kmax), C.byref(t))
        return self._finish(rid, rc, kmax, t)

    def wait(self, rid: int, timeout_s: float = 60.0):
        kmax, t = C.c_uint32(), L.ServeTiming()
        rc = lib().kc_serve_wait(self._h, rid, C.byref(kmax), C.byref(t), timeout_s)
        r = self._finish(rid, rc, kmax, t)
        if r is None:
            raise TimeoutError(f"request {rid} not done after {timeout_s} s")
        return r

    def stats(self) -> dict:
        st = L.ServeStats()
        check(lib().kc_serve_stats_get(self._h, C.byref(st)), "kc_serve_stats_get")
        return st.as_dict()

    def close(self) -> None:
        if getattr(self, "_h", None):
            rc = lib().kc_serve_close(self._h)
            self._h = None
            check(rc, "kc_serve_close")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
