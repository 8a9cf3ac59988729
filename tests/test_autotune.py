"""The autotuner's choices (kc_autotune) on the degree distributions of the
benchmark workloads and a few other shapes, on CPU: it reads a sample of the
host offsets only.  The GPU parity under every setting it can choose (and
under forced ones) is tests/test_modes_gpu.py."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import kcoregpu_gb300 as kc
from kcoregpu_gb300 import workloads as W

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("cfg,budget", [(1, 128), (2, 128), (3, 256)])
def test_single_graph_workloads(cfg, budget):
    t = kc.autotune(W.single_graph(cfg)[0])
    # skewed degrees: short warp-local cascades (longer above 2M vertices);
    # graphs above 256K vertices hand the last 16,384 survivors to the tail
    assert t == {"hub_arcs": 256, "chunk_arcs": 64, "local_budget": budget, "tail_v": 16384, "grid": 0}


def test_near_uniform_degrees_get_long_cascades():
    off = kc.build_csr(*kc.gen_er(300_000, 1_500_000, 79))[0]
    t = kc.autotune(off)
    assert t["local_budget"] == 512 and t["tail_v"] == 16384


def test_small_graph_hands_over_at_12288():
    off = kc.build_csr(*kc.gen_rmat(60_000, 500_000, 42))[0]
    assert kc.autotune(off)["tail_v"] == 12288


def test_empty_and_edgeless_graphs():
    assert kc.autotune(np.zeros(1, np.uint32))["chunk_arcs"] == 64
    assert kc.autotune(np.zeros(11, np.uint32))["local_budget"] == 512   # all degrees 0: no spread


def test_overrides_win():
    code = ("import sys; sys.path.insert(0, %r)\n"
            "import kcoregpu_gb300 as kc\n"
            "from kcoregpu_gb300 import workloads as W\n"
            "print(kc.autotune(W.single_graph(1)[0]))") % str(ROOT)
    env = {**os.environ, "KC_CHUNK_ARCS": "128", "KC_HUB_ARCS": "512", "KC_LOCAL_BUDGET": "64", "KC_TAIL_V": "0"}
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    t = eval(r.stdout.strip().splitlines()[-1])
    assert t == {"hub_arcs": 512, "chunk_arcs": 128, "local_budget": 64, "tail_v": 0, "grid": 0}
