"""Parity against the reference's own GPU build on the same GB300.

The reference's level-synchronous kernels (selectNodesAtLevel1 and
processNodes1, src/ours.cc + src/buffer.cc) are compiled unmodified into
oracle/_ref/ref_peel.cubin by oracle/build_ref.sh; oracle/ref_peel_driver.cpp
replays kcore()'s host loop (ours.cc:117-160) through the CUDA driver API and
writes the final degree array, which is the core numbers.  Our peel must give
the same core numbers and kmax, bit for bit.  The prebuilt reference cubin must be
present: a GPU run without it fails here instead of passing quietly.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import kcoregpu_gb300 as kc
from conftest import golden_names, golden_serialized

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
CUBIN = ROOT / "oracle" / "_ref" / "ref_peel.cubin"
DRIVER = ROOT / "oracle" / "_build" / "ref_peel_driver"


def _reference_peel(off, nbr, tmp: Path):
    assert CUBIN.exists(), f"the reference's kernels were not built ({CUBIN.name} missing): run oracle/build_ref.sh"
    assert DRIVER.exists(), f"{DRIVER.name} missing: build the oracle first"
    f = tmp / "csr.bin"
    with open(f, "wb") as fh:
        np.array([len(off) - 1, len(nbr)], np.uint32).tofile(fh)
        np.asarray(off, np.uint32).tofile(fh)
        np.asarray(nbr, np.uint32).tofile(fh)
    out = tmp / "core.bin"
    r = subprocess.run([str(DRIVER), str(CUBIN), str(f), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr or r.stdout
    tok = r.stdout.split()
    return np.fromfile(out, dtype=np.uint32), int(tok[tok.index("kmax") + 1])


def _graphs():
    gs = [(f"golden-{n}", *golden_serialized(n)[:2]) for n in golden_names()]
    gs += [
        ("er-20k", *kc.build_csr(*kc.gen_er(20_000, 100_000, 41))[:2]),
        ("rmat-60k", *kc.build_csr(*kc.gen_rmat(60_000, 500_000, 42))[:2]),
        ("chunglu-80k-g2.1", *kc.build_csr(*kc.gen_chung_lu(80_000, 300_000, 2.1, 8_000.0, 43))[:2]),
        ("rmat-400k-3.4M", *kc.build_csr(*kc.gen_rmat(400_000, 3_400_000, 1))[:2]),
    ]
    return gs


@pytest.mark.parametrize("name,off,nbr", [pytest.param(*g, id=g[0]) for g in _graphs()])
def test_same_core_numbers_as_the_reference_gpu_build(gpu, tmp_path, name, off, nbr):
    want, wk = _reference_peel(off, nbr, tmp_path)
    core, k = kc.peel_csr(off, nbr)
    np.testing.assert_array_equal(core, want[: len(off) - 1])
    assert k == wk
