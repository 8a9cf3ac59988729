"""TEST INFRASTRUCTURE ONLY: ctypes view of oracle/_build/libkc_oracle.so.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may import this
module; the product path never does.  Besides the CPU peels it exposes the
oracle's own workload generators and CSR builder (kc_gen_oracle.c), which the
reference arm of bench.py uses to make its input without the product library.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libkc_oracle.so"
_lib = None
_u32p = C.POINTER(C.c_uint32)
_u64p = C.POINTER(C.c_uint64)


def _load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            LIB.parent.mkdir(exist_ok=True)
            subprocess.run(["gcc", "-O2", "-std=gnu11", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared",
                            str(HERE / "kc_oracle.c"), str(HERE / "kc_gen_oracle.c"), "-o", str(LIB), "-lm"],
                           check=True)
        h = C.CDLL(str(LIB))
        h.kco_bz.restype = C.c_uint32
        h.kco_bz.argtypes = [C.c_uint32, _u32p, _u32p, _u32p]
        h.kco_levelsync.restype = C.c_uint32
        h.kco_levelsync.argtypes = [C.c_uint32, _u32p, _u32p, _u32p, _u32p, _u32p, C.c_uint32,
                                    C.c_int, _u32p]
        h.kco_batch_bz.restype = None
        h.kco_batch_bz.argtypes = [C.c_uint32, _u64p, _u64p, _u32p, _u32p, _u32p, _u32p, C.c_int]
        h.kco_num_threads.restype = C.c_int
        h.kco_gen_rmat.restype = C.c_int
        h.kco_gen_rmat.argtypes = [C.c_uint32, C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                   _u32p, _u32p]
        h.kco_gen_chung_lu.restype = C.c_int
        h.kco_gen_chung_lu.argtypes = [C.c_uint32, C.c_uint64, C.c_double, C.c_double, C.c_uint64, _u32p, _u32p]
        h.kco_gen_er.restype = C.c_int
        h.kco_gen_er.argtypes = [C.c_uint32, C.c_uint64, C.c_uint64, _u32p, _u32p]
        h.kco_build_csr.restype = C.c_int
        h.kco_build_csr.argtypes = [_u32p, _u32p, C.c_uint64, _u32p, _u64p, C.POINTER(_u32p), C.POINTER(_u32p)]
        h.kco_free.restype = None
        h.kco_free.argtypes = [C.c_void_p]
        h.kco_gen_batch.restype = C.c_int
        h.kco_gen_batch.argtypes = [C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, C.c_double, C.c_double,
                                    C.c_double, C.c_double, C.c_double, C.POINTER(_u64p), C.POINTER(_u64p),
                                    C.POINTER(_u32p), C.POINTER(_u32p)]
        _lib = h
    return _lib


def _p(a):
    return a.ctypes.data_as(_u32p)


def bz(offsets, neighbors):
    """Batagelj-Zaversnik core numbers -> (core, kmax)."""
    off = np.ascontiguousarray(offsets, np.uint32)
    nbr = np.ascontiguousarray(neighbors, np.uint32)
    V = len(off) - 1
    core = np.empty(max(V, 1), np.uint32)
    k = _load().kco_bz(V, _p(off), _p(nbr) if len(nbr) else None, _p(core))
    return core[:V], int(k)


def levelsync(offsets, neighbors, nthreads: int = 1, with_order: bool = False):
    """The reference's level-synchronous peel (src/ours.cc:117-160) on the host
    -> (core, kmax, levels[, order, shells])."""
    off = np.ascontiguousarray(offsets, np.uint32)
    nbr = np.ascontiguousarray(neighbors, np.uint32)
    V = len(off) - 1
    core = np.empty(max(V, 1), np.uint32)
    order = np.empty(max(V, 1), np.uint32) if with_order else None
    maxdeg = int(np.diff(off).max()) if V else 0
    shells = np.empty(maxdeg + 2, np.uint32) if with_order else None
    levels = C.c_uint32()
    k = _load().kco_levelsync(V, _p(off), _p(nbr) if len(nbr) else None, _p(core),
                              _p(order) if with_order else None,
                              _p(shells) if with_order else None,
                              len(shells) if with_order else 0, nthreads, C.byref(levels))
    if with_order:
        return core[:V], int(k), levels.value, order[:V], shells[: levels.value + 1]
    return core[:V], int(k), levels.value


def batch_bz(vbase, abase, offsets, neighbors, nthreads: int):
    """Per-graph BZ over a segmented CSR (OpenMP over graphs) -> (core, kmax[])."""
    vb = np.ascontiguousarray(vbase, np.uint64)
    ab = np.ascontiguousarray(abase, np.uint64)
    off = np.ascontiguousarray(offsets, np.uint32)
    nbr = np.ascontiguousarray(neighbors, np.uint32)
    ng = len(vb) - 1
    core = np.empty(max(int(vb[-1]), 1), np.uint32)
    kmax = np.empty(max(ng, 1), np.uint32)
    _load().kco_batch_bz(ng, vb.ctypes.data_as(_u64p), ab.ctypes.data_as(_u64p), _p(off), _p(nbr),
                         _p(core), _p(kmax), nthreads)
    return core[: int(vb[-1])], kmax[:ng]


def num_threads() -> int:
    return int(_load().kco_num_threads())


def _check(rc: int, what: str) -> None:
    if rc:
        raise RuntimeError(f"oracle {what} failed: {rc}")


def gen_rmat(n: int, n_edges: int, seed: int, a=0.57, b=0.19, c=0.19):
    """R-MAT draws (kc_gen_oracle.c) -> (src, dst)."""
    s = np.empty(max(n_edges, 1), np.uint32)
    t = np.empty(max(n_edges, 1), np.uint32)
    _check(_load().kco_gen_rmat(n, n_edges, a, b, c, seed, _p(s), _p(t)), "kco_gen_rmat")
    return s[:n_edges], t[:n_edges]


def gen_chung_lu(n: int, m: int, gamma: float, max_w: float, seed: int):
    """Chung-Lu pairs (kc_gen_oracle.c) -> (src, dst)."""
    s = np.empty(max(m, 1), np.uint32)
    t = np.empty(max(m, 1), np.uint32)
    _check(_load().kco_gen_chung_lu(n, m, gamma, max_w, seed, _p(s), _p(t)), "kco_gen_chung_lu")
    return s[:m], t[:m]


def gen_er(n: int, m: int, seed: int):
    """Erdos-Renyi G(n, m) pairs (kc_gen_oracle.c) -> (src, dst)."""
    s = np.empty(max(m, 1), np.uint32)
    t = np.empty(max(m, 1), np.uint32)
    _check(_load().kco_gen_er(n, m, seed, _p(s), _p(t)), "kco_gen_er")
    return s[:m], t[:m]


def build_csr(src, dst):
    """Reference CSR of directed pairs (graph.cpp:84-122 semantics) -> (offsets, neighbors)."""
    s = np.ascontiguousarray(src, np.uint32)
    t = np.ascontiguousarray(dst, np.uint32)
    V = C.c_uint32()
    E = C.c_uint64()
    po, pn = _u32p(), _u32p()
    h = _load()
    _check(h.kco_build_csr(_p(s) if len(s) else None, _p(t) if len(t) else None, len(s), C.byref(V), C.byref(E),
                           C.byref(po), C.byref(pn)), "kco_build_csr")
    try:
        off = np.ctypeslib.as_array(po, shape=(V.value + 1,)).copy()
        nbr = np.ctypeslib.as_array(pn, shape=(max(E.value, 1),))[: E.value].copy()
    finally:
        h.kco_free(C.cast(po, C.c_void_p))
        h.kco_free(C.cast(pn, C.c_void_p))
    return off, nbr


def gen_batch(ngraphs: int, seed_base: int, nmin: int, nmax: int, dmin: float, dmax: float,
              a=0.57, b=0.19, c=0.19):
    """The segmented batch (kc_gen_oracle.c) -> (vbase, abase, offsets, neighbors)."""
    vb, ab = _u64p(), _u64p()
    po, pn = _u32p(), _u32p()
    h = _load()
    _check(h.kco_gen_batch(ngraphs, seed_base, nmin, nmax, dmin, dmax, a, b, c, C.byref(vb), C.byref(ab),
                           C.byref(po), C.byref(pn)), "kco_gen_batch")
    try:
        vbase = np.ctypeslib.as_array(vb, shape=(ngraphs + 1,)).copy()
        abase = np.ctypeslib.as_array(ab, shape=(ngraphs + 1,)).copy()
        nv, na = int(vbase[-1]), int(abase[-1])
        off = np.ctypeslib.as_array(po, shape=(nv + ngraphs,)).copy()
        nbr = np.ctypeslib.as_array(pn, shape=(max(na, 1),))[:na].copy()
    finally:
        for p in (vb, ab, po, pn):
            h.kco_free(C.cast(p, C.c_void_p))
    return vbase, abase, off, nbr
