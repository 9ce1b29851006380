"""Build the synchrowords GB300 shared library (nvcc, sm_103a) in-tree.

Produces ``synchrowords_gb300/_build/libsynchrowords.so`` (the C ABI of
``include/synchrowords.h``) and ``synchrowords_gb300/_build/synchro`` (the
command-line drop-in).  Translation units are compiled in parallel; a unit is
rebuilt when its source or any header is newer than its object.
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
LIB = BUILD / "libsynchrowords.so"
CLI = BUILD / "synchro"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "-I", str(ROOT / "include")]

LIB_SOURCES = ["kernels.cu", "subset_check.cu", "noalloc.cu", "pairs.cu", "brute.cu", "batch_small.cu",
               "batch_cluster.cu", "mlp.cu",
               "learn.cu", "exact.cu", "plan.cpp", "automaton.cpp", "abi.cpp"]
CLI_SOURCES = ["cli.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build synchrowords_gb300")


def _newest_header() -> float:
    hs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + list((ROOT / "include").glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile(src: Path, obj: Path, extra: list[str]) -> None:
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [nvcc(), *NVCC_FLAGS, *extra, "-x", "c++", "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    extra = list(extra or [])
    hdr = _newest_header()
    objs = []
    jobs = []
    for name in LIB_SOURCES + CLI_SOURCES:
        src = CSRC / name
        obj = BUILD / (name.replace(".", "_") + ".o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr):
            jobs.append((src, obj))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            list(ex.map(lambda j: _compile(j[0], j[1], extra), jobs))
    lib_objs = [o for o, n in zip(objs, LIB_SOURCES + CLI_SOURCES) if n in LIB_SOURCES]
    cli_objs = [o for o, n in zip(objs, LIB_SOURCES + CLI_SOURCES) if n in CLI_SOURCES]
    if jobs or not LIB.exists():
        tmp = BUILD / f"libsynchrowords.{os.getpid()}.so"
        cmd = [nvcc(), *ARCH, "-shared", *map(str, lib_objs), "-o", str(tmp), "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stderr}")
        os.replace(tmp, LIB)
    if jobs or not CLI.exists():
        cmd = [nvcc(), *ARCH, *map(str, cli_objs), "-o", str(CLI), "-L", str(BUILD), "-lsynchrowords",
               "-Xlinker", "-rpath=$ORIGIN", "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
