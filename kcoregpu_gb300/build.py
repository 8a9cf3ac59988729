"""In-tree build of libkcore_gb300.so (sm_103a), the `kcore` CLI and the
oracle library used by the tests.

Every translation unit is compiled in parallel; the whole build takes well
under a minute and needs only nvcc, g++ and make-free Python.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
LIB = PKG / "libkcore_gb300.so"
CLI = PKG / "kcore"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "libkc_oracle.so"
ORACLE_SOURCES = ["kc_oracle.c", "kc_gen_oracle.c"]
ORACLE_CFLAGS = ["-O2", "-std=gnu11", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without floating-point contraction: the seeded
# generators then round every expression the same way on x86 and Arm hosts
# (Arm compilers would otherwise fuse a*b+c).
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-fopenmp,-O3,-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall", f"-I{INCLUDE}", f"-I{CSRC}"]

CU_SOURCES = ["kc_peel.cu", "kc_tail.cu", "kc_hindex.cu", "kc_hxtail.cu", "kc_validate.cu", "kc_api.cu", "kc_noalloc.cu", "kc_batch.cu", "kc_batch_host.cu",
              "kc_serve.cu"]
CXX_SOURCES = ["kc_host.cpp", "kc_gen.cpp"]
CHECKED_SOURCES = ["kc_peel.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src = CSRC / s
        if not src.exists():
            continue
        obj = BUILD / (s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)])
    for s in CHECKED_SOURCES:   # bounds-checked second instantiation (KC_CHECKED=1)
        src = CSRC / s
        obj = BUILD / (s + ".checked.o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + ["-DKC_CHECKED", "-c", str(src), "-o", str(obj)])
    for s in CXX_SOURCES:
        src = CSRC / s
        obj = BUILD / (s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] +
             ["-Xcompiler", "-fopenmp", "-lgomp"])
    cli_src = CSRC / "kcore_cli.cpp"
    if cli_src.exists() and (force or _stale(CLI, [cli_src, LIB] + headers)):
        _run(["g++"] + CXX_FLAGS + [str(cli_src), "-o", str(CLI), f"-L{PKG}", "-lkcore_gb300",
                                    f"-Wl,-rpath,$ORIGIN"])
    return LIB


def build_oracle(force: bool = False) -> Path:
    srcs = [ORACLE_DIR / s for s in ORACLE_SOURCES]
    ORACLE_LIB.parent.mkdir(exist_ok=True)
    if force or _stale(ORACLE_LIB, srcs):
        _run(["gcc"] + ORACLE_CFLAGS + [str(s) for s in srcs] + ["-o", str(ORACLE_LIB), "-lm"])
    # driver that replays the reference's host loop around its own kernels
    drv_src = ORACLE_DIR / "ref_peel_driver.cpp"
    drv = ORACLE_DIR / "_build" / "ref_peel_driver"
    cuda_inc = Path("/usr/local/cuda/include")
    if drv_src.exists() and (force or _stale(drv, [drv_src])):
        libdirs = [p for p in ("/usr/local/cuda/lib64/stubs", "/usr/local/cuda/lib64") if Path(p).exists()]
        _run(["g++", "-O2", "-std=c++17", f"-I{cuda_inc}", str(drv_src), "-o", str(drv)] +
             [f"-L{p}" for p in libdirs] + ["-lcuda"])
    return ORACLE_LIB


def build_reference_oracle() -> None:
    """Builds oracle/_ref from the reference sources when a reference checkout
    is present (KC_REFERENCE_DIR, else a `reference` directory beside this
    repository); without one nothing is built.  oracle/_ref is git-ignored: its
    files exist only in a working tree that was built next to the reference
    sources, and travel with that tree to a GPU host as files (the reference's
    kernels are a device-code cubin; its x86 loader binary does not run on an
    Arm host)."""
    script = ORACLE_DIR / "build_ref.sh"
    ref = os.environ.get("KC_REFERENCE_DIR") or str(ROOT.parent / "reference")
    if script.exists() and Path(ref, "src").is_dir():
        subprocess.run(["bash", str(script)], check=False, capture_output=True,
                       env=dict(os.environ, KC_REFERENCE_DIR=ref))


def build_all(force: bool = False) -> None:
    build_library(force)
    build_oracle(force)
    build_reference_oracle()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB)
