"""Host-side mirror of the reference's plugin surface for the peel path.

* ``Graph`` mirrors ``class Graph`` (inc/graph.h:7-23, src/graph.cpp): the
  SNAP-style loader with the serialized cache, and the core-number writer.
* ``kcore(g)`` mirrors ``int kcore(Graph&)`` (src/ours.cc:117-160): it peels
  on the GPU, sets ``g.kmax`` and returns the elapsed time in whole
  milliseconds, like the reference driver; the core numbers are kept in
  ``g.core`` (the reference computes them but never copies them back,
  ours.cc:154-155).
* ``DeviceGraph`` is the device-resident graph of the C ABI (kc_graph).
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

from . import _lib as L
from ._lib import KCoreError, check, lib, ptr, u32

OUTPUT_LOC = "./output/"   # inc/common.h:17


def load_edgelist(path: str, parse_mode: str = "snap"):
    """Graph::readFile (graph.cpp:58-124) -> (offsets, neighbors, degrees)."""
    c = L.CsrHost()
    check(lib().kc_load_edgelist(os.fsencode(path), L.PARSE_MODES[parse_mode], C.byref(c)),
          "kc_load_edgelist")
    return L.csr_to_numpy(c)


def build_csr(src, dst):
    """Reference CSR semantics (graph.cpp:84-122) from a directed edge array."""
    s, t = u32(src), u32(dst)
    if len(s) != len(t):
        raise ValueError("src and dst differ in length")
    c = L.CsrHost()
    check(lib().kc_build_csr(ptr(s), ptr(t), len(s), C.byref(c)), "kc_build_csr")
    return L.csr_to_numpy(c)


def read_serialized(path: str):
    c = L.CsrHost()
    check(lib().kc_read_serialized(os.fsencode(path), C.byref(c)), "kc_read_serialized")
    return L.csr_to_numpy(c)


def write_serialized(path: str, offsets, neighbors, degrees=None) -> None:
    off, nbr = u32(offsets), u32(neighbors)
    deg = u32(np.diff(off)) if degrees is None else u32(degrees)
    c = L.numpy_to_csr(off, nbr, deg)
    check(lib().kc_write_serialized(os.fsencode(path), C.byref(c)), "kc_write_serialized")


def read_csr_binary(path: str):
    """Binary CSR sidecar -> (offsets, neighbors, degrees)."""
    c = L.CsrHost()
    check(lib().kc_read_csr_binary(os.fsencode(path), C.byref(c)), "kc_read_csr_binary")
    return L.csr_to_numpy(c)


def write_csr_binary(path: str, offsets, neighbors) -> None:
    off, nbr = u32(offsets), u32(neighbors)
    c = L.numpy_to_csr(off, nbr, u32(np.diff(off)))
    check(lib().kc_write_csr_binary(os.fsencode(path), C.byref(c)), "kc_write_csr_binary")


def write_core_json(path: str, core) -> None:
    """Graph::writeKCoreToDisk bytes (graph.cpp:126-140)."""
    c = u32(core)
    check(lib().kc_write_core_json(os.fsencode(path), ptr(c), len(c)), "kc_write_core_json")


def write_core_txt(path: str, core) -> None:
    c = u32(core)
    check(lib().kc_write_core_txt(os.fsencode(path), ptr(c), len(c)), "kc_write_core_txt")


def write_edgelist(path: str, src, dst) -> None:
    s, t = u32(src), u32(dst)
    check(lib().kc_write_edgelist(os.fsencode(path), ptr(s), ptr(t), len(s)), "kc_write_edgelist")


def gen_rmat(n: int, n_edges: int, seed: int, a=0.57, b=0.19, c=0.19):
    s = np.empty(n_edges, np.uint32)
    t = np.empty(n_edges, np.uint32)
    check(lib().kc_gen_rmat(n, n_edges, a, b, c, seed, ptr(s), ptr(t)), "kc_gen_rmat")
    return s, t


def gen_chung_lu(n: int, m: int, gamma: float, max_w: float, seed: int):
    m = min(m, n * (n - 1) // 2)
    s = np.empty(m, np.uint32)
    t = np.empty(m, np.uint32)
    check(lib().kc_gen_chung_lu(n, m, gamma, max_w, seed, ptr(s), ptr(t)), "kc_gen_chung_lu")
    return s, t


def gen_er(n: int, m: int, seed: int):
    m = min(m, n * (n - 1) // 2)
    s = np.empty(m, np.uint32)
    t = np.empty(m, np.uint32)
    check(lib().kc_gen_er(n, m, seed, ptr(s), ptr(t)), "kc_gen_er")
    return s, t


def autotune(offsets) -> dict:
    """The autotuner's settings for a CSR (kc_autotune): hub threshold, task
    chunk, cascade budget, tail hand-off point, grid."""
    off = u32(offsets)
    t = L.Tuning()
    check(lib().kc_autotune(ptr(off), len(off) - 1, C.byref(t)), "kc_autotune")
    return t.as_dict()


def device_info() -> dict:
    sms, grid, ma, mi = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    check(lib().kc_device_info(C.byref(sms), C.byref(grid), C.byref(ma), C.byref(mi)), "kc_device_info")
    return {"sms": sms.value, "grid": grid.value, "cc": f"{ma.value}.{mi.value}"}


class DeviceGraph:
    """A CSR resident in HBM with its peel state (C ABI kc_graph)."""

    def __init__(self, offsets, neighbors, method: str = "auto"):
        self.offsets = u32(offsets)
        self.neighbors = u32(neighbors)
        self.V = len(self.offsets) - 1
        h = C.c_void_p()
        nb = ptr(self.neighbors) if len(self.neighbors) else None
        check(lib().kc_graph_upload(ptr(self.offsets), nb, self.V, C.byref(h)), "kc_graph_upload")
        self._h = h
        if method != "auto":
            self.set_method(method)

    @property
    def handle(self):
        return self._h

    METHODS = {"auto": 0, "hindex": 1, "peel": 2}

    def set_method(self, method: str) -> None:
        """'auto' (the process default), 'hindex' (the h-index fixed point, the
        level peel after KC_HX_ITERS iterations without convergence) or 'peel'
        (the level-synchronous peel).  The core numbers are the same."""
        check(lib().kc_graph_set_method(self._h, self.METHODS[method]), "kc_graph_set_method")

    def set_stream(self, stream_handle: int | None) -> None:
        check(lib().kc_graph_set_stream(self._h, C.c_void_p(stream_handle or 0)), "kc_graph_set_stream")

    def peel_async(self) -> None:
        check(lib().kc_graph_peel_async(self._h), "kc_graph_peel_async")

    def fetch(self, want_core: bool = True):
        core = np.empty(self.V, np.uint32) if want_core else None
        kmax = C.c_uint32()
        st = L.Stats()
        check(lib().kc_graph_fetch(self._h, ptr(core) if want_core and self.V else None,
                                   C.byref(kmax), C.byref(st)), "kc_graph_fetch")
        return core, kmax.value, st.as_dict()

    def peel(self):
        """-> (core numbers, kmax, stats)"""
        core = np.empty(self.V, np.uint32)
        kmax = C.c_uint32()
        st = L.Stats()
        check(lib().kc_peel(self._h, ptr(core) if self.V else None, C.byref(kmax), C.byref(st)), "kc_peel")
        return core, kmax.value, st.as_dict()

    def degeneracy_order(self):
        """-> (order, shell_offsets, kmax): vertices in peel order and the
        k-shell boundaries (kcore-global-buffer/KCore.h:244-272)."""
        maxdeg = int(np.diff(self.offsets).max()) if self.V else 0
        order = np.empty(max(self.V, 1), np.uint32)
        shells = np.empty(maxdeg + 2, np.uint32)
        kmax = C.c_uint32()
        check(lib().kc_degeneracy_order(self._h, ptr(order), ptr(shells), len(shells), C.byref(kmax)),
              "kc_degeneracy_order")
        k = kmax.value
        nsh = 1 if self.V == 0 else k + 2
        return order[: self.V], shells[:nsh], k

    def trace(self):
        """Per-level device trace -> (levels x 8) uint64 array: level start,
        CTA 0 arrival, level complete, CTA 0 saw completion (ns), vertices
        peeled so far, last CTA arrival (ns), walk rounds and adjacency quads
        walked (levels of the one-CTA tail kernel; 0 for grid levels)."""
        maxdeg = int(np.diff(self.offsets).max()) if self.V else 0
        buf = np.zeros((maxdeg + 2) * 8, np.uint64)
        lv = C.c_uint32()
        check(lib().kc_graph_trace(self._h, buf.ctypes.data_as(C.POINTER(C.c_uint64)), maxdeg + 2,
                                   C.byref(lv)), "kc_graph_trace")
        return buf.reshape(-1, 8)[: lv.value]

    def free(self) -> None:
        if getattr(self, "_h", None):
            lib().kc_graph_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def peel_csr(offsets, neighbors):
    """One-shot peel of a host CSR -> (core numbers, kmax)."""
    off, nbr = u32(offsets), u32(neighbors)
    V = len(off) - 1
    core = np.empty(V, np.uint32)
    kmax = C.c_uint32()
    check(lib().kc_peel_csr(ptr(off), ptr(nbr) if len(nbr) else None, V, ptr(core) if V else None,
                            C.byref(kmax)), "kc_peel_csr")
    return core, kmax.value


class Graph:
    """Mirror of the reference's Graph (inc/graph.h:7-23)."""

    def __init__(self, input_file: str | None = None, cache_dir: str = OUTPUT_LOC,
                 parse_mode: str = "snap"):
        self.V = 0
        self.E = 0
        self.neighbors = np.zeros(0, np.uint32)
        self.neighbors_offset = np.zeros(1, np.uint32)
        self.degrees = np.zeros(0, np.uint32)
        self.kmax = 0
        self.core = None
        self.from_cache = False
        self.cache_kind = 0   # 1: text serialized cache, 2: its binary sidecar
        self.cache_dir = cache_dir
        self.parse_mode = parse_mode
        if input_file is not None:
            # Graph::Graph(path): serialized cache first, else parse + write it
            # (graph.cpp:142-154).
            c = L.CsrHost()
            hit = C.c_int()
            check(lib().kc_load_graph(os.fsencode(input_file), os.fsencode(cache_dir),
                                      L.PARSE_MODES[parse_mode], C.byref(c), C.byref(hit)),
                  "kc_load_graph")
            self._set(*L.csr_to_numpy(c))
            self.from_cache = bool(hit.value)
            self.cache_kind = hit.value

    def _set(self, off, nbr, deg):
        self.neighbors_offset, self.neighbors, self.degrees = off, nbr, deg
        self.V = len(off) - 1
        self.E = int(off[-1]) if len(off) else 0

    @classmethod
    def from_csr(cls, offsets, neighbors) -> "Graph":
        g = cls()
        off, nbr = u32(offsets), u32(neighbors)
        g._set(off, nbr, u32(np.diff(off)))
        return g

    @classmethod
    def from_edges(cls, src, dst) -> "Graph":
        g = cls()
        g._set(*build_csr(src, dst))
        return g

    def readFile(self, input_file: str) -> None:
        self._set(*load_edgelist(input_file, self.parse_mode))

    def readSerialized(self, input_file: str) -> bool:
        path = os.path.join(self.cache_dir, "serialized-" + os.path.basename(input_file))
        if not os.path.exists(path):
            return False
        self._set(*read_serialized(path))
        return True

    def writeSerialized(self, input_file: str) -> None:
        path = os.path.join(self.cache_dir, "serialized-" + os.path.basename(input_file))
        if os.path.isdir(self.cache_dir):
            write_serialized(path, self.neighbors_offset, self.neighbors, self.degrees)

    def writeKCoreToDisk(self, file: str) -> None:
        """Writes <cache_dir>/pkc-kcore-<file> from the core numbers when a peel
        ran (else from degrees, which is what the reference writes)."""
        vals = self.core if self.core is not None else self.degrees
        write_core_json(os.path.join(self.cache_dir, "pkc-kcore-" + file), vals)


def kcore(g: Graph) -> int:
    """int kcore(Graph&) (src/ours.cc:117-160): GPU peel of g; sets g.kmax and
    g.core; returns elapsed whole milliseconds of the peel."""
    t0 = time.perf_counter()
    core, kmax = peel_csr(g.neighbors_offset, g.neighbors)
    ms = int((time.perf_counter() - t0) * 1000.0)
    g.kmax = kmax
    g.core = core
    return ms
