"""Build recipe for the compiled reference (test infrastructure, not product).

Compiles SynchroLib 1.1.0's own sources, read where they lie under the
reference checkout, into a binary under ``oracle/_ref/`` (git-ignored).  Only
the tests, the smoke check and bench.py's CPU-baseline leg run the result,
and only as a checker / baseline.

The reference normally JIT-compiles itself per (N, K): it copies its tree,
substitutes ``$DEFINES$`` / ``$EXACT_DEF$`` ... tokens with ``#define`` lines
built from the JSON plan (app/jit.hpp:17-141, jitlib/jitlib.hpp:124-196,
synchrolib/algorithm/*/config.hpp) and runs make.  Every such token sits in an
``#ifndef __INTELLISENSE__`` block except the one in jit/jitdefines.hpp, so
this recipe instead compiles the untouched sources with ``-D__INTELLISENSE__``
and puts its own generated ``jitdefines.hpp`` first on the include path.  The
generated defines follow the reference's config-to-define mapping
(algorithm/config.hpp:13-55 and each algorithm's config.hpp); values that are
C++ expressions (``"AUT_N * 16"``) are passed through verbatim, exactly as the
reference does, so the C++ compiler evaluates them.

The reference's ``run()`` plugin entry (jit/jitmain.cpp:11-49) is linked with
oracle/ref_driver.cpp, which stands in for app/main.cpp.

Usage:  python oracle/build_ref.py N K plan.json [--threads T]
prints the path of the built binary.  Needs g++ and the reference checkout;
builds are cached by (N, K, defines).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import hashlib
import json
import os
import subprocess
import sys
from pathlib import Path

REF_ROOT = Path(os.environ.get("SYNCHRO_REF_ROOT", "/root/reference"))
HERE = Path(__file__).resolve().parent
OUT_ROOT = HERE / "_ref"

# Translation units of the reference's JIT library (jit/makefile_jit:6).
REF_SOURCES = [
    "jit/jitmain.cpp",
    "synchrolib/algorithm/exact/exact.cpp",
    "synchrolib/algorithm/exact/meet_in_the_middle.cpp",
    "synchrolib/algorithm/exact/dfs.cpp",
    "synchrolib/data_structures/preprocessed_transitions.cpp",
    "synchrolib/utils/distribution.cpp",
    "synchrolib/utils/connectivity.cpp",
]

DEFAULT_UPPER_BOUND = "1ULL * AUT_N * AUT_N * AUT_N / 6"  # app/jit.hpp:152


def _str_int(cfg: dict, key: str, default: str) -> str:
    """algorithm/config.hpp:26-35 (get_str_int)."""
    if key not in cfg:
        return default
    v = cfg[key]
    return v if isinstance(v, str) else str(int(v))


def _str_bool(cfg: dict, key: str, default: str) -> str:
    """algorithm/config.hpp:36-45 (get_str_bool)."""
    if key not in cfg:
        return default
    v = cfg[key]
    return v if isinstance(v, str) else ("true" if v else "false")


def _str_float(cfg: dict, key: str, default: str) -> str:
    """algorithm/config.hpp:46-55 (get_str_float; std::to_string prints %f)."""
    if key not in cfg:
        return default
    v = cfg[key]
    return v if isinstance(v, str) else "%f" % float(v)


def _define(name: str, value: str | None = None) -> str:
    """algorithm/config.hpp:13-15 (make_define wraps the value in parentheses)."""
    return f"#define {name}" + ("" if not value else f" ({value})") + "\n"


def algorithm_defines(name: str, cfg: dict) -> str:
    """Per-algorithm defines, one function per reference config class."""
    out = ""
    if name == "Exact":  # algorithm/exact/config.hpp:24-46
        out += _define("DFS_SHORTCUT", _str_bool(cfg, "dfs_shortcut", "true"))
        out += _define("DFS", _str_bool(cfg, "dfs", "true"))
        out += _define("STRICT_MEMORY_LIMIT", _str_bool(cfg, "strict_memory_limit", "false"))
        out += _define("MAX_MEMORY", _str_int(cfg, "max_memory_mb", "2048"))
        out += _define("DFS_MIN_LIST_SIZE", _str_int(cfg, "dfs_min_list_size", "10000"))
        out += _define("BFS_SMALL_LIST_SIZE", _str_int(cfg, "bfs_small_list_size", "AUT_N * 16"))
    elif name == "Beam":  # algorithm/beam/config.hpp:23-44
        out += _define("BEAM_SIZE", _str_int(cfg, "beam_size", "std::log2(AUT_N)"))
        out += _define("DYNAMIC", _str_bool(cfg, "dynamic", "false"))
        out += _define("MIN_BEAM_SIZE", _str_int(cfg, "min_beam_size", "AUT_N * std::log2(AUT_N)"))
        out += _define("MAX_BEAM_SIZE", _str_int(cfg, "max_beam_size", "AUT_N * AUT_N * std::log2(AUT_N)"))
        out += _define("BEAM_EXACT_RATIO", _str_float(cfg, "beam_exact_ratio", "0.01"))
        out += _define("MAX_ITER", _str_int(cfg, "max_iter", "-1"))
        presort = cfg.get("presort", "none")
        if presort not in ("none", "indeg"):
            raise ValueError("presort value not in [none, indeg]")
        out += _define("PRESORT_" + presort.upper())
    elif name == "Brute":  # algorithm/brute/config.hpp:23-26
        out += _define("MAX_N", _str_int(cfg, "max_n", "20"))
    elif name == "Eppstein":  # algorithm/eppstein/config.hpp:23-31
        out += _define("TRANSITION_TABLES", _str_bool(cfg, "transition_tables", "false"))
        out += _define("FIND_WORD", _str_bool(cfg, "find_word", "false"))
    elif name == "Reduce":  # algorithm/reduce/config.hpp:24-32
        out += _define("MIN_N", _str_int(cfg, "min_n", "80"))
        out += _define("LIST_SIZE_THRESHOLD", _str_int(cfg, "list_size_threshold", "AUT_N * 16"))
    else:
        raise ValueError("Unknown algorithm: " + name)
    return out


def jit_defines(plan: dict, n: int, k: int, threads: int | None = None) -> str:
    """app/jit.hpp:112-141 (get_global_defines) plus the algorithm defines."""
    t = int(plan.get("threads", 1) if threads is None else threads)
    if t < 1 or t > 64:
        raise ValueError("threads must belong to range [1, 64]")
    s = "#pragma once\n"
    s += _define("AUT_N", str(n)) + _define("AUT_K", str(k))
    s += _define("UPPER_BOUND", _str_int(plan, "upper_bound", DEFAULT_UPPER_BOUND))
    s += _define("GPU", "false")  # the reference's CUDA path does not build with CUDA 13
    s += _define("GPU_MEMORY", _str_int(plan, "gpu_max_memory_mb", "1024 * 2"))
    s += _define("THREADS", str(t))
    s += _define("JIT")
    names = sorted({a["name"] for a in plan["algorithms"]})
    for name in names:
        s += _define("COMPILE_" + name.upper())
    for a in plan["algorithms"]:
        s += algorithm_defines(a["name"], a.get("config", {}) or {})
    return s


def build(n: int, k: int, plan: dict, threads: int | None = None, verbose: bool = False) -> Path:
    if not REF_ROOT.is_dir():
        raise FileNotFoundError(f"reference checkout not found at {REF_ROOT}")
    defines = jit_defines(plan, n, k, threads)
    algos = ",".join(a["name"] for a in plan["algorithms"])
    tag = hashlib.sha1((defines + algos).encode()).hexdigest()[:12]
    out_dir = OUT_ROOT / f"synchro_{n}_{k}_{tag}"
    binary = out_dir / "synchro_ref"
    if binary.exists():
        return binary
    gen = out_dir / "gen"
    gen.mkdir(parents=True, exist_ok=True)
    (gen / "jitdefines.hpp").write_text(defines)
    # Flags of jit/makefile_jit:2 (minus -s/-fPIC, plus the INTELLISENSE guard).
    flags = ["-std=c++17", "-Ofast", "-march=native", "-flto", "-DNDEBUG", "-pthread",
             "-D__INTELLISENSE__", "-w", f"-I{gen}", f"-I{REF_ROOT}"]
    jobs = []
    for src in REF_SOURCES:
        obj = out_dir / (src.replace("/", "_") + ".o")
        jobs.append(["g++", *flags, "-c", str(REF_ROOT / src), "-o", str(obj)])
    drv_obj = out_dir / "ref_driver.o"
    jobs.append(["g++", *flags, f'-DREF_ALGORITHMS="{algos}"', "-c",
                 str(HERE / "ref_driver.cpp"), "-o", str(drv_obj)])
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, results):
        if r.returncode != 0:
            raise RuntimeError("reference build failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])
    objs = [j[-1] for j in jobs]
    r = subprocess.run(["g++", "-std=c++17", "-Ofast", "-march=native", "-flto", "-pthread",
                        *objs, "-o", str(binary)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference link failed:\n" + r.stderr[-4000:])
    return binary


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("n", type=int)
    ap.add_argument("k", type=int)
    ap.add_argument("plan")
    ap.add_argument("--threads", type=int, default=None)
    a = ap.parse_args()
    plan = json.loads(Path(a.plan).read_text())
    print(build(a.n, a.k, plan, a.threads))


if __name__ == "__main__":
    sys.exit(main())
