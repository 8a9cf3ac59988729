"""Batched peel: many independent graphs in one persistent launch (C ABI
kc_batch_*), plus the batch generator.  No reference counterpart: the
reference peels one graph per process (main.cu:44-91)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import check, lib, ptr, u32

_u64p = C.POINTER(C.c_uint64)
_u32p = C.POINTER(C.c_uint32)


SegCsr = L.SegCsr
BatchStats = L.BatchStats


class Segmented:
    """A segmented CSR: graph g has V_g = vbase[g+1]-vbase[g] vertices, local
    offsets offsets[vbase[g]+g : vbase[g]+g+V_g+1] and local neighbour ids
    neighbors[abase[g]:abase[g+1]]."""

    def __init__(self, vbase, abase, offsets, neighbors, owner=None):
        self.vbase = np.ascontiguousarray(vbase, np.uint64)
        self.abase = np.ascontiguousarray(abase, np.uint64)
        self.offsets = offsets if owner is not None else u32(offsets)
        self.neighbors = neighbors if owner is not None else u32(neighbors)
        self._owner = owner   # library allocation backing the arrays (kc_gen_batch)

    @property
    def ngraphs(self) -> int:
        return len(self.vbase) - 1

    @classmethod
    def from_graphs(cls, graphs) -> "Segmented":
        """Packs [(offsets, neighbors), ...] (graph-local ids)."""
        vb, ab = [0], [0]
        for off, nbr in graphs:
            vb.append(vb[-1] + len(off) - 1)
            ab.append(ab[-1] + len(nbr))
        offs = np.concatenate([u32(o) for o, _ in graphs]) if graphs else np.zeros(0, np.uint32)
        nbrs = np.concatenate([u32(n) for _, n in graphs]) if graphs else np.zeros(0, np.uint32)
        return cls(vb, ab, offs, nbrs)

    def graph(self, g: int):
        v0, v1 = int(self.vbase[g]), int(self.vbase[g + 1])
        a0, a1 = int(self.abase[g]), int(self.abase[g + 1])
        return self.offsets[v0 + g: v1 + g + 1], self.neighbors[a0:a1]

    def c_struct(self) -> SegCsr:
        s = SegCsr()
        s.ngraphs = self.ngraphs
        s.vbase = self.vbase.ctypes.data_as(_u64p)
        s.abase = self.abase.ctypes.data_as(_u64p)
        s.offsets = ptr(self.offsets) if len(self.offsets) else None
        s.neighbors = ptr(self.neighbors) if len(self.neighbors) else None
        return s


class _GenOwner:
    def __init__(self, s: SegCsr):
        self.s = s

    def __del__(self):
        try:
            lib().kc_segcsr_free(C.byref(self.s))
        except Exception:
            pass


def gen_batch(ngraphs: int, seed_base: int, nmin: int = 1000, nmax: int = 200000,
              dmin: float = 4.0, dmax: float = 32.0, a=0.57, b=0.19, c=0.19) -> Segmented:
    """Graph g: seed seed_base+g, n ~ log-uniform[nmin,nmax], average degree
    2m/n ~ U[dmin,dmax]; even g Erdos-Renyi, odd g R-MAT (a,b,c)."""
    s = SegCsr()
    check(lib().kc_gen_batch(ngraphs, seed_base, nmin, nmax, dmin, dmax, a, b, c, C.byref(s)), "kc_gen_batch")
    owner = _GenOwner(s)
    G = s.ngraphs
    vb = np.ctypeslib.as_array(s.vbase, shape=(G + 1,))
    ab = np.ctypeslib.as_array(s.abase, shape=(G + 1,))
    offs = np.ctypeslib.as_array(s.offsets, shape=(int(vb[-1]) + G,))
    nbrs = np.ctypeslib.as_array(s.neighbors, shape=(max(int(ab[-1]), 1),))[: int(ab[-1])]
    return Segmented(vb, ab, offs, nbrs, owner=owner)


class Batch:
    """A segmented CSR resident in HBM (C ABI kc_batch)."""

    def __init__(self, seg: Segmented):
        self.seg = seg
        h = C.c_void_p()
        check(lib().kc_batch_upload(C.byref(seg.c_struct()), C.byref(h)), "kc_batch_upload")
        self._h = h

    def set_stream(self, stream_handle: int | None) -> None:
        check(lib().kc_batch_set_stream(self._h, C.c_void_p(stream_handle or 0)), "kc_batch_set_stream")

    def peel_async(self) -> None:
        check(lib().kc_batch_peel_async(self._h), "kc_batch_peel_async")

    def fetch(self, want_core: bool = True):
        V = int(self.seg.vbase[-1])
        core = np.empty(max(V, 1), np.uint32) if want_core else None
        kmax = np.empty(max(self.seg.ngraphs, 1), np.uint32)
        st = BatchStats()
        check(lib().kc_batch_fetch(self._h, ptr(core) if want_core else None, ptr(kmax), C.byref(st)),
              "kc_batch_fetch")
        return (core[:V] if want_core else None), kmax[: self.seg.ngraphs], st.as_dict()

    def peel(self):
        """-> (core numbers of all graphs, per-graph kmax, stats)"""
        self.peel_async()
        return self.fetch()

    def peel_per_graph(self) -> float:
        """The one-graph-per-launch baseline; returns its device ms."""
        ms = C.c_float()
        check(lib().kc_batch_peel_per_graph(self._h, C.byref(ms)), "kc_batch_peel_per_graph")
        return ms.value

    def plan(self):
        G = self.seg.ngraphs
        sched = np.empty(max(G, 1), np.uint32)
        ng, qc, bl = C.c_uint32(), C.c_uint32(), C.c_uint32()
        check(lib().kc_batch_plan(self._h, ptr(sched), C.byref(ng), C.byref(qc), C.byref(bl)), "kc_batch_plan")
        return {"schedule": sched[:G], "giants": ng.value, "qcap": qc.value, "blocks": bl.value}

    def free(self) -> None:
        if getattr(self, "_h", None):
            lib().kc_batch_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
