"""The h-index peel (kcoregpu_gb300/csrc/kc_hindex.cu) against the oracle.

The h-index fixed point is the default method of a graph (kc_graph_set_method
selects per graph, KC_ALGO=peel|hindex sets the process default): it runs
first when no peel order or trace is asked for, and the level peel runs only
when it gives up (KC_HX_ITERS iterations, default 256).  The core numbers must equal the oracle's bit for
bit either way, and `stats["method"]` says which one produced them (1 =
h-index).  Shapes: hubs far above the chunk size (windows narrowed over
several passes), cliques and bipartite cores (every estimate falls together),
paths and cycles (one hop per iteration), isolated vertices, random R-MAT,
Chung-Lu and Erdos-Renyi graphs, and raw CSRs with duplicate arcs and
self-loops (compared with the reference's level-synchronous algorithm, which
counts each arc).  Child processes pin the process default and the
fallback: by default the one-shot entry goes through the h-index,
KC_HX_ITERS=2 stops it early and the level peel finishes, KC_ALGO=peel makes
the level peel the default, and a graph set to the level peel runs it alone.
"""
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import kcoregpu_gb300 as kc
from oracle import kc_oracle as O

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def _sym(s, t, n=None):
    return kc.build_csr(np.asarray(s, np.uint32), np.asarray(t, np.uint32))[:2]


def star(n):
    return _sym(np.zeros(n), np.arange(1, n + 1))


def clique(n):
    i, j = np.triu_indices(n, 1)
    return _sym(i, j)


def bipartite(a, b):
    i, j = np.meshgrid(np.arange(a), np.arange(a, a + b))
    return _sym(i.ravel(), j.ravel())


def path(n):
    s = np.arange(n - 1)
    return _sym(s, s + 1)


def cycle(n):
    s = np.arange(n)
    return _sym(s, (s + 1) % n)


def stars_and_cliques():
    # hubs joined to a clique: windows must narrow from 50K down to the clique's core
    parts, base = [], 0
    s_all, t_all = [], []
    for hub_leaves in (50_000, 20_000, 3_000):
        s_all.append(np.full(hub_leaves, base)); t_all.append(np.arange(base + 1, base + 1 + hub_leaves))
        base += hub_leaves + 1
    k = 300
    i, j = np.triu_indices(k, 1)
    s_all.append(i + base); t_all.append(j + base)
    hubs = [0, 50_001, 70_002]
    for h in hubs:   # each hub also joins the whole clique
        s_all.append(np.full(k, h)); t_all.append(np.arange(base, base + k))
    return _sym(np.concatenate(s_all), np.concatenate(t_all))


SHAPES = {
    "star-200k": lambda: star(200_000),
    "clique-400": lambda: clique(400),
    "bipartite-300x500": lambda: bipartite(300, 500),
    "stars+clique": stars_and_cliques,
    "cycle-100": lambda: cycle(100),
    "rmat-200k": lambda: kc.build_csr(*kc.gen_rmat(200_000, 1_600_000, seed=11))[:2],
    "rmat-64k-dense": lambda: kc.build_csr(*kc.gen_rmat(1 << 16, 2_000_000, seed=5))[:2],
    "chunglu-300k": lambda: kc.build_csr(*kc.gen_chung_lu(300_000, 1_200_000, 2.1, 30_000.0, seed=12))[:2],
    "chunglu-100k-g25": lambda: kc.build_csr(*kc.gen_chung_lu(100_000, 600_000, 2.5, 5_000.0, seed=3))[:2],
    "er-50k": lambda: kc.build_csr(*kc.gen_er(50_000, 300_000, seed=13))[:2],
}


@pytest.mark.parametrize("name", sorted(SHAPES))
def test_hindex_matches_oracle(gpu, name):
    off, nbr = SHAPES[name]()
    want, wk = O.bz(off, nbr)
    g = kc.DeviceGraph(off, nbr, method="hindex")
    for _ in range(3):   # repeated runs reuse every list and slot
        core, kmax, st = g.peel()
        np.testing.assert_array_equal(core, want)
        assert kmax == wk and st["levels"] == wk + 1
        assert st["method"] == 1, st
    g.free()


def test_isolated_vertices_and_tiny_graphs(gpu):
    for off, nbr in [(np.array([0, 0, 0, 0], np.uint32), np.array([], np.uint32)),
                     _sym([0], [1]), _sym([0, 1], [1, 2])]:
        want, wk = O.bz(off, nbr)
        core, kmax, st = kc.DeviceGraph(off, nbr, method="hindex").peel()
        np.testing.assert_array_equal(core, want)
        assert kmax == wk


def test_duplicate_arcs_and_self_loops_follow_the_reference_rule(gpu):
    # a raw CSR: every arc counts, a self-loop never decrements its own vertex
    rng = np.random.default_rng(4)
    V = 3000
    s0 = rng.integers(0, V, 20_000).astype(np.uint32)
    t0 = rng.integers(0, V, 20_000).astype(np.uint32)
    loops = np.arange(0, V, 7, dtype=np.uint32)
    s = np.concatenate([s0, t0, loops])   # both directions, repeats kept, plus self-loops
    t = np.concatenate([t0, s0, loops])
    order = np.lexsort((t, s))
    s, t = s[order], t[order]
    off = np.zeros(V + 1, np.uint32)
    np.add.at(off, s + 1, 1)
    off = np.cumsum(off).astype(np.uint32)
    nbr = t.astype(np.uint32)
    want, wk, _, _, _ = O.levelsync(off, nbr, nthreads=1, with_order=True)
    core, kmax, st = kc.DeviceGraph(off, nbr, method="hindex").peel()
    np.testing.assert_array_equal(core, want)
    assert kmax == wk and st["method"] == 1


def test_path_falls_back_to_the_level_peel(gpu):
    # a 5,000-vertex path needs about 2,500 h-index iterations: the level peel
    # finishes it after the default 256
    off, nbr = path(5_000)
    want, wk = O.bz(off, nbr)
    core, kmax, st = kc.DeviceGraph(off, nbr, method="hindex").peel()
    np.testing.assert_array_equal(core, want)
    assert kmax == wk and st["method"] == 0


def _child(code, **env):
    e = dict(os.environ)
    for k in ("KC_ALGO", "KC_HX_ITERS", "KC_HX_HANDOFF", "KC_HX_HO_FRONT", "KC_HX_HO_N", "KC_HX_TAIL_ITERS"):
        e.pop(k, None)
    e.update({k: str(v) for k, v in env.items()})
    pre = f"import sys, json; sys.path.insert(0, {str(ROOT)!r})\nimport numpy as np\nimport kcoregpu_gb300 as kc\nfrom oracle import kc_oracle as O\n"
    r = subprocess.run([sys.executable, "-c", pre + code], capture_output=True, text=True, timeout=600, env=e, cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


CHILD = """
res = {}
for name, (off, nbr) in {
        'chunglu': kc.build_csr(*kc.gen_chung_lu(300_000, 1_200_000, 2.1, 30_000.0, seed=12))[:2],
        'rmat': kc.build_csr(*kc.gen_rmat(200_000, 1_600_000, seed=11))[:2]}.items():
    want, wk = O.bz(off, nbr)
    out = []
    for method in ('auto', 'peel'):
        g = kc.DeviceGraph(off, nbr, method=method)
        core, kmax, st = g.peel()
        out.append([bool(np.array_equal(core, want) and kmax == wk), int(st['method'])])
        g.free()
    core, kmax = kc.peel_csr(off, nbr)   # one-shot entry: the process default, CSR checked on the device
    out.append(bool(np.array_equal(core, want) and kmax == wk))
    res[name] = out
print(json.dumps(res))
"""


def test_process_default_is_hindex_and_one_shot_entry(gpu):
    out = _child(CHILD)
    assert out == {"chunglu": [[True, 1], [True, 0], True], "rmat": [[True, 1], [True, 0], True]}


def test_early_stop_hands_over_to_the_level_peel(gpu):
    out = _child(CHILD, KC_HX_ITERS=2)
    assert out == {"chunglu": [[True, 0], [True, 0], True], "rmat": [[True, 0], [True, 0], True]}


def test_level_peel_as_process_default(gpu):
    out = _child(CHILD, KC_ALGO="peel")
    assert out == {"chunglu": [[True, 0], [True, 0], True], "rmat": [[True, 0], [True, 0], True]}


@pytest.mark.parametrize("cfg", [1, 2, 3])
def test_benchmark_workloads_converge_by_hindex(gpu, cfg):
    from kcoregpu_gb300 import workloads
    off, nbr = workloads.single_graph(cfg)
    want, wk = O.bz(off, nbr)
    g = kc.DeviceGraph(off, nbr, method="hindex")
    core, kmax, st = g.peel()
    np.testing.assert_array_equal(core, want)
    assert kmax == wk and st["method"] == 1 and st["iterations"] <= 256
    g.free()
