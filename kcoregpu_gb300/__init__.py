"""kcoregpu_gb300 - GB300-native k-core decomposition (level-synchronous peel).

Python view of the C ABI in include/kcore.h (libkcore_gb300.so).  The compute
path is the sm_103a CUDA library; importing works without a GPU, and every
peel raises KCoreError(KC_ERR_NODEV) when no device is present.
"""
from ._lib import KCoreError, lib  # noqa: F401
from .graph import (  # noqa: F401
    DeviceGraph, Graph, autotune, build_csr, device_info, gen_chung_lu, gen_er, gen_rmat, kcore,
    load_edgelist, peel_csr, read_csr_binary, read_serialized, write_core_json, write_core_txt,
    write_csr_binary, write_edgelist, write_serialized,
)
