"""TEST INFRASTRUCTURE ONLY: ctypes view of oracle/_build/libkc_oracle.so.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may import this
module; the product path never does.
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
            subprocess.run(["gcc", "-O2", "-std=c11", "-fPIC", "-fopenmp", "-shared",
                            str(HERE / "kc_oracle.c"), "-o", str(LIB)], check=True)
        h = C.CDLL(str(LIB))
        h.kco_bz.restype = C.c_uint32
        h.kco_bz.argtypes = [C.c_uint32, _u32p, _u32p, _u32p]
        h.kco_levelsync.restype = C.c_uint32
        h.kco_levelsync.argtypes = [C.c_uint32, _u32p, _u32p, _u32p, _u32p, _u32p, C.c_uint32,
                                    C.c_int, _u32p]
        h.kco_batch_bz.restype = None
        h.kco_batch_bz.argtypes = [C.c_uint32, _u64p, _u64p, _u32p, _u32p, _u32p, _u32p, C.c_int]
        h.kco_num_threads.restype = C.c_int
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
