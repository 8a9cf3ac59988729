"""ctypes binding of libkcore_gb300.so (declared in include/kcore.h).

The product path is the CUDA library; there is no CPU fallback.  Loading
fails loudly when the in-tree library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libkcore_gb300.so"

KC_OK = 0
ERRORS = {
    -1: "KC_ERR_IO", -2: "KC_ERR_PARSE", -3: "KC_ERR_OOM", -4: "KC_ERR_OVERFLOW",
    -5: "KC_ERR_TIMEOUT", -6: "KC_ERR_CUDA", -7: "KC_ERR_BUDGET", -8: "KC_ERR_INVALID",
    -9: "KC_ERR_NODEV", -10: "KC_ERR_BUSY", -11: "KC_ERR_CLOSED",
}
PARSE_MODES = {"snap": 0, "reference": 1}


class KCoreError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str = ""):
        self.code = code
        self.name = ERRORS.get(code, str(code))
        super().__init__(f"{where}: {self.name}" + (f" ({msg})" if msg else ""))


class CsrHost(C.Structure):
    _fields_ = [("V", C.c_uint32), ("E", C.c_uint32), ("offsets", C.POINTER(C.c_uint32)),
                ("neighbors", C.POINTER(C.c_uint32)), ("degrees", C.POINTER(C.c_uint32))]


class Stats(C.Structure):
    _fields_ = [("V", C.c_uint32), ("kmax", C.c_uint32), ("levels", C.c_uint32),
                ("iterations", C.c_uint32), ("blocks", C.c_uint32), ("arcs", C.c_uint64), ("tasks", C.c_uint64),
                ("peel_ms", C.c_float), ("total_ms", C.c_float), ("method", C.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_u32p = C.POINTER(C.c_uint32)
_u64p = C.POINTER(C.c_uint64)
_vp = C.c_void_p
_cp = C.c_char_p


class SegCsr(C.Structure):
    _fields_ = [("ngraphs", C.c_uint32), ("vbase", _u64p), ("abase", _u64p),
                ("offsets", _u32p), ("neighbors", _u32p)]


class ServeCfg(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("ring_slots", C.c_uint32), ("gang_arcs", C.c_uint32),
                ("max_gang", C.c_uint32), ("small_vertices", C.c_uint32)]


class ServeTiming(C.Structure):
    _fields_ = [("queue_us", C.c_double), ("latency_us", C.c_double), ("gang", C.c_uint32),
                ("iterations", C.c_uint32), ("copy_in_us", C.c_double), ("peel_us", C.c_double),
                ("copy_out_us", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServeStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("in_use", C.c_uint64),
                ("peak_in_use", C.c_uint64), ("pending", C.c_uint32), ("inflight", C.c_uint32),
                ("blocks", C.c_uint32), ("direct", C.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tuning(C.Structure):
    _fields_ = [("hub_arcs", C.c_uint32), ("chunk_arcs", C.c_uint32), ("local_budget", C.c_uint32),
                ("tail_v", C.c_uint32), ("grid", C.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchStats(C.Structure):
    _fields_ = [("ngraphs", C.c_uint32), ("giants", C.c_uint32), ("blocks", C.c_uint32),
                ("qcap", C.c_uint32), ("V_total", C.c_uint64), ("arcs_total", C.c_uint64),
                ("peel_ms", C.c_float)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}

# name -> (restype, argtypes); every entry is declared in include/kcore.h
SIGNATURES = {
    "kc_strerror": (C.c_char_p, [C.c_int]),
    "kc_last_error": (C.c_char_p, []),
    "kc_device_info": (C.c_int, [C.POINTER(C.c_int)] * 4),
    "kc_host_alloc": (_vp, [C.c_size_t]),
    "kc_host_free": (None, [_vp]),
    "kc_load_edgelist": (C.c_int, [_cp, C.c_int, C.POINTER(CsrHost)]),
    "kc_build_csr": (C.c_int, [_u32p, _u32p, C.c_uint64, C.POINTER(CsrHost)]),
    "kc_csr_free": (None, [C.POINTER(CsrHost)]),
    "kc_read_serialized": (C.c_int, [_cp, C.POINTER(CsrHost)]),
    "kc_write_serialized": (C.c_int, [_cp, C.POINTER(CsrHost)]),
    "kc_read_csr_binary": (C.c_int, [_cp, C.POINTER(CsrHost)]),
    "kc_write_csr_binary": (C.c_int, [_cp, C.POINTER(CsrHost)]),
    "kc_load_graph": (C.c_int, [_cp, _cp, C.c_int, C.POINTER(CsrHost), C.POINTER(C.c_int)]),
    "kc_write_core_json": (C.c_int, [_cp, _u32p, C.c_uint32]),
    "kc_write_core_txt": (C.c_int, [_cp, _u32p, C.c_uint32]),
    "kc_gen_rmat": (C.c_int, [C.c_uint32, C.c_uint64, C.c_double, C.c_double, C.c_double,
                              C.c_uint64, _u32p, _u32p]),
    "kc_gen_chung_lu": (C.c_int, [C.c_uint32, C.c_uint64, C.c_double, C.c_double, C.c_uint64,
                                  _u32p, _u32p]),
    "kc_gen_er": (C.c_int, [C.c_uint32, C.c_uint64, C.c_uint64, _u32p, _u32p]),
    "kc_write_edgelist": (C.c_int, [_cp, _u32p, _u32p, C.c_uint64]),
    "kc_graph_upload": (C.c_int, [_u32p, _u32p, C.c_uint32, C.POINTER(_vp)]),
    "kc_graph_set_stream": (C.c_int, [_vp, _vp]),
    "kc_graph_set_method": (C.c_int, [_vp, C.c_uint32]),
    "kc_graph_peel_async": (C.c_int, [_vp]),
    "kc_graph_fetch": (C.c_int, [_vp, _u32p, _u32p, C.POINTER(Stats)]),
    "kc_peel": (C.c_int, [_vp, _u32p, _u32p, C.POINTER(Stats)]),
    "kc_degeneracy_order": (C.c_int, [_vp, _u32p, _u32p, C.c_uint32, _u32p]),
    "kc_graph_trace": (C.c_int, [_vp, _u64p, C.c_uint32, _u32p]),
    "kc_graph_device_ptrs": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp)]),
    "kc_graph_free": (None, [_vp]),
    "kc_peel_csr": (C.c_int, [_u32p, _u32p, C.c_uint32, _u32p, _u32p]),
    "kc_autotune": (C.c_int, [_u32p, C.c_uint32, C.POINTER(Tuning)]),
    "kc_peel_noalloc": (C.c_int, [_vp, _vp, C.c_uint32, C.c_uint32, _vp, _u32p, _vp]),
    "kc_batch_upload": (C.c_int, [C.POINTER(SegCsr), C.POINTER(_vp)]),
    "kc_batch_set_stream": (C.c_int, [_vp, _vp]),
    "kc_batch_peel_async": (C.c_int, [_vp]),
    "kc_batch_fetch": (C.c_int, [_vp, _u32p, _u32p, C.POINTER(BatchStats)]),
    "kc_batch_peel_per_graph": (C.c_int, [_vp, C.POINTER(C.c_float)]),
    "kc_batch_plan": (C.c_int, [_vp, _u32p, _u32p, _u32p, _u32p]),
    "kc_batch_free": (None, [_vp]),
    "kc_batch_peel": (C.c_int, [C.POINTER(SegCsr), _u32p, _u32p, C.POINTER(BatchStats)]),
    "kc_gen_batch": (C.c_int, [C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, C.c_double, C.c_double,
                               C.c_double, C.c_double, C.c_double, C.POINTER(SegCsr)]),
    "kc_segcsr_free": (None, [C.POINTER(SegCsr)]),
    "kc_serve_open": (C.c_int, [C.POINTER(ServeCfg), C.POINTER(_vp)]),
    "kc_serve_submit": (C.c_int, [_vp, _u32p, _u32p, C.c_uint32, _u32p, _u64p]),
    "kc_serve_poll": (C.c_int, [_vp, C.c_uint64, _u32p, C.POINTER(ServeTiming)]),
    "kc_serve_wait": (C.c_int, [_vp, C.c_uint64, _u32p, C.POINTER(ServeTiming), C.c_double]),
    "kc_serve_stats_get": (C.c_int, [_vp, C.POINTER(ServeStats)]),
    "kc_serve_close": (C.c_int, [_vp]),
    "kc_serve_debug": (C.c_int, [_vp, _u64p, C.c_uint32]),
}

_lib = None


def lib() -> C.CDLL:
    """Loads the in-tree CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: run kcoregpu_gb300.build.build_all() first")
        h = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
    return _lib


def check(rc: int, where: str) -> None:
    if rc != KC_OK:
        msg = lib().kc_last_error()
        raise KCoreError(rc, where, msg.decode() if msg else "")


def u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def ptr(a: np.ndarray):
    return a.ctypes.data_as(_u32p)


def csr_to_numpy(c: CsrHost) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Copies a library-owned CSR into numpy arrays and frees it."""
    V, E = int(c.V), int(c.E)
    off = np.ctypeslib.as_array(c.offsets, shape=(V + 1,)).copy() if c.offsets else np.zeros(1, np.uint32)
    nbr = np.ctypeslib.as_array(c.neighbors, shape=(E,)).copy() if (c.neighbors and E) else np.zeros(0, np.uint32)
    deg = np.ctypeslib.as_array(c.degrees, shape=(V,)).copy() if (c.degrees and V) else np.zeros(0, np.uint32)
    lib().kc_csr_free(C.byref(c))
    return off, nbr, deg


def numpy_to_csr(off: np.ndarray, nbr: np.ndarray, deg: np.ndarray) -> CsrHost:
    c = CsrHost()
    c.V = len(off) - 1
    c.E = len(nbr)
    c.offsets = ptr(off)
    c.neighbors = ptr(nbr) if len(nbr) else None
    c.degrees = ptr(deg) if len(deg) else None
    return c


def num_threads() -> int:
    return os.cpu_count() or 1
