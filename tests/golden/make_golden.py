"""Regenerates the golden fixtures in this directory.

Inputs are small edge lists made here with numpy (seeded) plus hand-written
known-answer graphs.  Expected outputs come from two independent sources:

* the reference's own loader and writer (src/graph.cpp, built unmodified into
  oracle/_ref/ref_loader by oracle/build_ref.sh): ``serialized-<name>`` (the CSR
  cache bytes, graph.cpp:35-54) and ``pkc-kcore-<name>`` (writeKCoreToDisk bytes,
  graph.cpp:126-140);
* networkx.core_number on the same graph: ``<name>.core`` ("v core" per vertex),
  the check the reference's verification notebook makes.

Run from the repository root on the build host:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import tempfile
from pathlib import Path

import networkx as nx
import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REF_LOADER = ROOT / "oracle" / "_ref" / "ref_loader"

KNOWN = {
    # name: edge-list text (no comment or blank lines: the reference loader
    # reads such lines as edges, graph.cpp:86-88)
    "triangle_tail": "0 1\n1 2\n2 0\n2 3\n",
    "k5": "".join(f"{i} {j}\n" for i in range(5) for j in range(i + 1, 5)),
    "star8": "".join(f"0 {i}\n" for i in range(1, 9)),
    "path10": "".join(f"{i} {i + 1}\n" for i in range(9)),
    "isolated_ids": "3 7\n7 9\n9 3\n12 3\n",
    "self_loops_only": "4 4\n2 2\n",
    "duplicates": "1 2\n2 1\n1 2\n2 3\n3 2\n3 1\n1 3\n",
    "two_cliques": "".join(f"{i} {j}\n" for i in range(6) for j in range(i + 1, 6)) +
                   "".join(f"{i} {j}\n" for i in range(10, 14) for j in range(i + 1, 14)) + "5 10\n",
    "tabs_crlf": "0\t1\r\n1\t2\r\n2\t0\r\n",
    "single_edge": "0 1\n",
}


def random_graphs() -> dict[str, str]:
    out = {}
    rng = np.random.default_rng(20240601)
    for i, (n, m) in enumerate([(40, 90), (200, 900), (1000, 6000), (2500, 20000)]):
        s = rng.integers(0, n, m)
        t = rng.integers(0, n, m)
        out[f"er_{n}"] = "".join(f"{a} {b}\n" for a, b in zip(s, t))
    # skewed: preferential endpoints (heavy tail) with duplicates and self-loops
    for n, m in [(300, 3000), (3000, 30000)]:
        w = 1.0 / np.arange(1, n + 1) ** 0.9
        w /= w.sum()
        s = rng.choice(n, m, p=w)
        t = rng.choice(n, m, p=w)
        out[f"skew_{n}"] = "".join(f"{a}\t{b}\n" for a, b in zip(s, t))
    return out


# Lines the reference reads in its own odd way (graph.cpp:86-88): a '#' line
# after a valid line becomes edge (0, previous t), a blank line repeats the
# previous edge, a letter-led line is skipped.
QUIRKS = {
    "quirk_hash_blank": "1 2\n# comment\n3 4\n\n5 6\nheader line\n7 8\n",
}


def nx_cores(off: np.ndarray, nbr: np.ndarray) -> np.ndarray:
    V = len(off) - 1
    G = nx.Graph()
    G.add_nodes_from(range(V))
    src = np.repeat(np.arange(V), np.diff(off))
    G.add_edges_from(zip(src.tolist(), nbr.tolist()))
    cn = nx.core_number(G)
    return np.array([cn[v] for v in range(V)], dtype=np.uint32)


def parse_serialized(p: Path):
    toks = p.read_text().split()
    V, E = int(toks[0]), int(toks[1])
    deg = np.array(toks[2:2 + V], dtype=np.uint64).astype(np.uint32)
    off = np.array(toks[2 + V:3 + 2 * V], dtype=np.uint64).astype(np.uint32)
    nbr = np.array(toks[3 + 2 * V:3 + 2 * V + E], dtype=np.uint64).astype(np.uint32)
    return off, nbr, deg


def main() -> None:
    if not REF_LOADER.exists():
        raise SystemExit("build oracle/_ref first: bash oracle/build_ref.sh")
    graphs = {**KNOWN, **random_graphs(), **QUIRKS}
    manifest = {}
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        (tmp / "output").mkdir()
        for name, text in graphs.items():
            src = HERE / f"{name}.txt"
            src.write_text(text)
            shutil.copy(src, tmp / f"{name}.txt")
            r = subprocess.run([str(REF_LOADER), "load", f"{name}.txt"], cwd=tmp, capture_output=True,
                               text=True)
            if r.returncode != 0:
                raise SystemExit(f"reference loader failed on {name}: {r.stderr}")
            ser = tmp / "output" / f"serialized-{name}.txt"
            shutil.copy(ser, HERE / f"serialized-{name}.txt")
            off, nbr, _ = parse_serialized(ser)
            core = nx_cores(off, nbr)
            (HERE / f"{name}.core").write_text("".join(f"{v} {c}\n" for v, c in enumerate(core.tolist())))
            (tmp / "core.txt").write_text(" ".join(map(str, core.tolist())))
            r = subprocess.run([str(REF_LOADER), "json", f"{name}.txt", "core.txt"], cwd=tmp,
                               capture_output=True, text=True)
            if r.returncode != 0:
                raise SystemExit(f"reference writer failed on {name}: {r.stderr}")
            shutil.copy(tmp / "output" / f"pkc-kcore-{name}.txt", HERE / f"pkc-kcore-{name}.txt")
            manifest[name] = {"V": int(len(off) - 1), "arcs": int(len(nbr)),
                              "kmax": int(core.max()) if len(core) else None,
                              "quirk": name in QUIRKS}
    (HERE / "manifest.json").write_text(json.dumps(manifest, indent=1, sort_keys=True) + "\n")
    print(f"wrote {len(manifest)} fixtures")


if __name__ == "__main__":
    os.chdir(ROOT)
    main()
