"""Shared fixtures.  `-m gpu` tests need a CUDA device and fail loudly
without one; everything else runs on CPU."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: full-size workloads")


@pytest.fixture(scope="session", autouse=True)
def built_library():
    from kcoregpu_gb300 import build
    build.build_library()
    build.build_oracle()
    return build.LIB


def golden_names(include_quirks: bool = False) -> list[str]:
    man = json.loads((GOLDEN / "manifest.json").read_text())
    return sorted(k for k, v in man.items() if include_quirks or not v["quirk"])


def golden_serialized(name: str):
    toks = (GOLDEN / f"serialized-{name}.txt").read_text().split()
    V, E = int(toks[0]), int(toks[1])
    deg = np.array(toks[2:2 + V], dtype=np.uint64).astype(np.uint32)
    off = np.array(toks[2 + V:3 + 2 * V], dtype=np.uint64).astype(np.uint32)
    nbr = np.array(toks[3 + 2 * V:3 + 2 * V + E], dtype=np.uint64).astype(np.uint32)
    return off, nbr, deg


def golden_core(name: str) -> np.ndarray:
    rows = [l.split() for l in (GOLDEN / f"{name}.core").read_text().splitlines() if l.strip()]
    return np.array([int(c) for _, c in rows], dtype=np.uint32)


@pytest.fixture(scope="session")
def gpu():
    """The CUDA device; fails (does not skip) when none is present."""
    import kcoregpu_gb300 as kc
    info = kc.device_info()
    return info
