"""GPU parity of the one-graph peel under each of its runtime settings.

The level-peel settings are run with KC_ALGO=peel (the h-index peel, which
runs first by default, would otherwise solve these graphs before the level
peel starts); KC_ALGO=hindex runs the h-index peel, and KC_HX_ITERS=3 stops
it early so that the level peel finishes from scratch; KC_HX_START=8 starts
the h-index after a level peel has left at most V/8 survivors (with
KC_HX_ITERS=2 the level peel then starts over).  The h-index peel hands its
last iterations to the cluster kernel by default: KC_HX_HANDOFF=0 keeps them
in the grid, KC_HX_HO_FRONT=10^9 tries the hand-off from the third iteration
on (large sets, failed certificates, later retries), KC_HX_HO_N=512 allows
only small sets, with KC_HX_TAIL_ITERS=2 the cluster gives up and the level
peel runs from the start, and KC_TAIL_V=0 (no level-peel tail buffers) leaves
the hand-off, which has buffers of its own, in place.  With KC_TAIL=hindex
the survivors handed to the tail go to the cluster h-index tail (16-CTA
cluster, estimates in distributed shared memory); with KC_HX_TAIL_ITERS=2 it
gives up and the level tail finishes them.
The settings are read once per process (KC_CLAIM_CAS: claim by CAS or read
the state first; KC_TAIL_V: the tail hand-off point, 0 = the persistent
kernel peels every level; KC_LOCAL_BUDGET: the cascade budget, its minimum
sending most cascades through the task queue; KC_HUB_ARCS and KC_CHUNK_ARCS:
the hub threshold and the task chunk the autotuner otherwise picks), so each
case runs in a fresh process.  Every case must give the oracle's core numbers and kmax, through
both the one-shot entry (kc_peel_csr) and a resident graph peeled twice."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]

CHILD = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, sys.argv[1] + "/tests")
import kcoregpu_gb300 as kc
from oracle import kc_oracle as O
graphs = [
    kc.build_csr(*kc.gen_rmat(60_000, 500_000, 42))[:2],
    kc.build_csr(*kc.gen_chung_lu(80_000, 300_000, 2.1, 8_000.0, 43))[:2],
    kc.build_csr(*kc.gen_er(20_000, 100_000, 41))[:2],
    kc.build_csr(*kc.gen_rmat(400_000, 3_400_000, 1))[:2],
]
for off, nbr in graphs:
    want, wk = O.bz(off, nbr)
    core, k = kc.peel_csr(off, nbr)
    assert np.array_equal(core, want) and k == wk, "peel_csr differs"
    g = kc.DeviceGraph(off, nbr)
    for _ in range(2):
        core, k, _ = g.peel()
        assert np.array_equal(core, want) and k == wk, "resident peel differs"
    g.free()
print("ok")
"""


LEVEL_PEEL = [
    {"KC_CLAIM_CAS": "0"},
    {"KC_TAIL_V": "0"},
    {"KC_TAIL_V": "16384"},
    {"KC_TAIL_V": "8192"},
    {"KC_LOCAL_BUDGET": "32"},
    {"KC_LOCAL_BUDGET": "4096"},
    {"KC_HUB_ARCS": "32"},
    {"KC_HUB_ARCS": "4096"},
    {"KC_CHUNK_ARCS": "256"},
    {"KC_CHUNK_ARCS": "100"},
    {"KC_CLAIM_CAS": "0", "KC_TAIL_V": "0", "KC_LOCAL_BUDGET": "32"},
    {"KC_HUB_ARCS": "32", "KC_CHUNK_ARCS": "64", "KC_LOCAL_BUDGET": "32"},
]


@pytest.mark.parametrize("env", [{"KC_ALGO": "peel", **e} for e in LEVEL_PEEL] +
                         [{"KC_ALGO": "hindex"}, {"KC_ALGO": "hindex", "KC_HX_ITERS": "3"},
                          {"KC_HX_START": "8"}, {"KC_HX_START": "8", "KC_HX_ITERS": "2"},
                          {"KC_HX_HANDOFF": "0"}, {"KC_HX_HO_FRONT": "1000000000"}, {"KC_TAIL_V": "0"},
                          {"KC_HX_HO_FRONT": "1000000000", "KC_HX_HO_N": "512"},
                          {"KC_HX_HO_FRONT": "1000000000", "KC_HX_TAIL_ITERS": "2"},
                          {"KC_ALGO": "peel", "KC_TAIL": "hindex"},
                          {"KC_ALGO": "peel", "KC_TAIL": "hindex", "KC_HX_TAIL_ITERS": "2"}],
                         ids=lambda e: ",".join(f"{k}={v}" for k, v in e.items()))
def test_peel_under_each_setting(gpu, env):
    r = subprocess.run([sys.executable, "-c", CHILD, str(ROOT)], env={**os.environ, **env},
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stderr[-2000:] or r.stdout[-2000:]
