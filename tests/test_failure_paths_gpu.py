"""Failure paths of the single-graph peel on the GPU, in forms that fault and
hang nothing: each runs in a fresh child process with a test-only setting read
once at start-up.  The wait and queue cases are those of the level peel, so
they run with KC_ALGO=peel (the h-index peel that runs first by default
solves these graphs without the task queue).

* KC_WAIT_US=50 shortens every device wait of the peel to 50 us.  On a
  300,000-vertex path one warp walks the whole level-1 cascade while the others
  wait for it, so their waits run out: the call returns KC_ERR_TIMEOUT (where
  the reference would spin in `while(count < V)`, src/ours.cc:138), and the
  same process then peels a batch bit for bit (the context stays usable).  A
  fresh process with the default limit peels the path bit for bit.
* KC_TASK_CAP=8 leaves the task queue room for 8 entries: a 200,000-leaf
  star, whose hub is claimed in level 1 and queues its adjacency as 782 tasks,
  returns KC_ERR_OVERFLOW (where the reference's queue overflow is an assert
  trap, src/buffer.cc:2), and the process again peels a batch bit for bit.
* KC_CHECKED=1 runs the bounds-checked kernel (every global and shared index
  checked; a violation would be recorded and the access skipped): adversarial
  shapes and random graphs through the three single-graph entry points give
  the oracle's core numbers with no violation recorded.
"""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]

PRELUDE = f"""
import json, sys
sys.path.insert(0, {str(ROOT)!r})
import numpy as np
import kcoregpu_gb300 as kc
from kcoregpu_gb300 import batch as B
from oracle import kc_oracle as O

def path(n):
    s = np.arange(n - 1, dtype=np.uint32)
    return kc.build_csr(s, s + 1)[:2]

def batch_ok():
    seg = B.Segmented.from_graphs([kc.build_csr(*kc.gen_rmat(3000, 20000, seed=7))[:2],
                                   kc.build_csr(*kc.gen_er(2000, 9000, seed=8))[:2]])
    core, kmax, _ = B.Batch(seg).peel()
    want, wk = O.batch_bz(seg.vbase, seg.abase, seg.offsets, seg.neighbors, 4)
    return bool(np.array_equal(core, want) and np.array_equal(kmax, wk))

def try_peel(off, nbr):
    try:
        g = kc.DeviceGraph(off, nbr)
        core, kmax, _ = g.peel()
        want, wk = O.bz(off, nbr)
        return "ok" if (np.array_equal(core, want) and kmax == wk) else "mismatch"
    except kc.KCoreError as e:
        return e.name
"""


def _child(code: str, **env) -> dict:
    e = dict(os.environ)
    for k in ("KC_WAIT_US", "KC_TASK_CAP", "KC_CHECKED", "KC_ALGO"):
        e.pop(k, None)
    e.update({k: str(v) for k, v in env.items()})
    r = subprocess.run([sys.executable, "-c", PRELUDE + code], capture_output=True, text=True, timeout=600, env=e,
                       cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_a_wait_that_runs_out_returns_timeout(gpu):
    out = _child("print(json.dumps({'path': try_peel(*path(300_000)), 'batch': batch_ok()}))", KC_WAIT_US=50,
                 KC_ALGO="peel")
    assert out == {"path": "KC_ERR_TIMEOUT", "batch": True}
    out = _child("print(json.dumps({'path': try_peel(*path(300_000))}))", KC_ALGO="peel")
    assert out == {"path": "ok"}


def test_a_full_task_queue_returns_overflow(gpu):
    code = ("s = np.zeros(200_000, np.uint32); t = np.arange(1, 200_001, dtype=np.uint32)\n"
            "off, nbr = kc.build_csr(s, t)[:2]\n"
            "print(json.dumps({'hubs': try_peel(off, nbr), 'batch': batch_ok()}))")
    assert _child(code, KC_TASK_CAP=8, KC_ALGO="peel") == {"hubs": "KC_ERR_OVERFLOW", "batch": True}


def test_bounds_checked_kernel_records_no_violation(gpu):
    code = """
import ctypes as C, torch
def star(n):
    s = np.zeros(n, np.uint32); t = np.arange(1, n + 1, dtype=np.uint32)
    return kc.build_csr(s, t)[:2]
def clique(n):
    i, j = np.triu_indices(n, 1)
    return kc.build_csr(i.astype(np.uint32), j.astype(np.uint32))[:2]
graphs = {'star-200k': star(200_000), 'clique-400': clique(400), 'path-100k': path(100_000),
          'rmat-200k': kc.build_csr(*kc.gen_rmat(200_000, 1_600_000, seed=11))[:2],
          'chunglu-300k': kc.build_csr(*kc.gen_chung_lu(300_000, 1_200_000, 2.1, 30_000.0, seed=12))[:2],
          'er-50k': kc.build_csr(*kc.gen_er(50_000, 300_000, seed=13))[:2]}
res = {}
for name, (off, nbr) in graphs.items():
    want, wk = O.bz(off, nbr)
    r = [try_peel(off, nbr)]
    try:
        core, k = kc.peel_csr(off, nbr)
        r.append('ok' if np.array_equal(core, want) and k == wk else 'mismatch')
    except kc.KCoreError as e:
        r.append(e.name)
    if len(off) - 1 <= 524288 and len(nbr) <= 8388608:
        d_off = torch.from_numpy(off.view(np.int32)).cuda(); d_nbr = torch.from_numpy(nbr.view(np.int32)).cuda()
        d_core = torch.empty(len(off) - 1, dtype=torch.int32, device='cuda'); km = C.c_uint32()
        rc = kc.lib().kc_peel_noalloc(C.c_void_p(d_off.data_ptr()), C.c_void_p(d_nbr.data_ptr()), len(off) - 1,
                                      len(nbr), C.c_void_p(d_core.data_ptr()), C.byref(km), None)
        got = d_core.cpu().numpy().view(np.uint32)
        r.append('ok' if rc == 0 and np.array_equal(got, want) and km.value == wk else f'rc{rc}')
    res[name] = r
print(json.dumps(res))
"""
    out = _child(code, KC_CHECKED=1)
    assert out and all(v == ["ok"] * len(v) for v in out.values()), out
