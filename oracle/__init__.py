"""ORACLE — test infrastructure, not product.

ctypes front end of the CPU restatement in oracle/oracle.cpp (SynchroLib's
Exact and Beam algorithms) plus helpers around the compiled reference
(oracle/build_ref.py).  Only tests/, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg may import this package, and only as the
checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field
from pathlib import Path
from typing import Optional, Sequence

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"


def build(force: bool = False) -> Path:
    """Compile oracle.cpp into oracle/_build/liboracle.so (g++, portable flags)."""
    src = HERE / "oracle.cpp"
    hdr = HERE / "oracle.h"
    if (not force and LIB.exists() and LIB.stat().st_mtime >= src.stat().st_mtime
            and LIB.stat().st_mtime >= hdr.stat().st_mtime):
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = BUILD / f"liboracle.{os.getpid()}.so"
    subprocess.run(["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-pthread",
                    str(src), "-o", str(tmp)], check=True)
    os.replace(tmp, LIB)
    return LIB


class _Bounds(ctypes.Structure):
    _fields_ = [("non_synchro", ctypes.c_int32), ("lower", ctypes.c_uint64), ("upper", ctypes.c_uint64)]


class _ExactParams(ctypes.Structure):
    _fields_ = [("dfs", ctypes.c_int32), ("dfs_shortcut", ctypes.c_int32),
                ("strict_memory_limit", ctypes.c_int32), ("max_memory_mb", ctypes.c_uint64),
                ("dfs_min_list_size", ctypes.c_uint64), ("bfs_small_list_size", ctypes.c_uint64),
                ("threads", ctypes.c_uint32)]


class _BeamParams(ctypes.Structure):
    _fields_ = [("beam_size", ctypes.c_uint64), ("dynamic", ctypes.c_int32),
                ("min_beam_size", ctypes.c_uint64), ("max_beam_size", ctypes.c_uint64),
                ("beam_exact_ratio", ctypes.c_double), ("max_iter", ctypes.c_int64),
                ("presort_indeg", ctypes.c_int32)]


class _TraceStep(ctypes.Structure):
    _fields_ = [("phase", ctypes.c_int32), ("novisited", ctypes.c_int32), ("len", ctypes.c_uint64),
                ("list_bfs", ctypes.c_uint64), ("list_invbfs", ctypes.c_uint64)]


class _Trace(ctypes.Structure):
    _fields_ = [("steps", ctypes.POINTER(_TraceStep)), ("capacity", ctypes.c_uint64),
                ("count", ctypes.c_uint64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build()))
        _lib.oracle_exact.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint32, ctypes.c_uint32,
                                      ctypes.POINTER(_ExactParams), ctypes.POINTER(_Bounds),
                                      ctypes.POINTER(_Trace)]
        _lib.oracle_beam.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint32, ctypes.c_uint32,
                                     ctypes.POINTER(_BeamParams), ctypes.POINTER(_Bounds)]
        _lib.oracle_brute.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint32, ctypes.c_uint32,
                                      ctypes.POINTER(ctypes.c_int64)]
        _lib.oracle_eppstein.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint32, ctypes.c_uint32,
                                         ctypes.POINTER(_Bounds), ctypes.POINTER(ctypes.c_uint32),
                                         ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]
    return _lib


@dataclass
class ExactParams:
    """Evaluated Exact defines; defaults are algorithm/exact/config.hpp:24-46 at a given n."""
    dfs: bool = True
    dfs_shortcut: bool = True
    strict_memory_limit: bool = False
    max_memory_mb: int = 2048
    dfs_min_list_size: int = 10000
    bfs_small_list_size: Optional[int] = None  # default AUT_N * 16
    threads: int = 1


@dataclass
class BeamParams:
    """Evaluated Beam defines (algorithm/beam/config.hpp:23-44); None = reference default."""
    beam_size: Optional[int] = None
    dynamic: bool = False
    min_beam_size: Optional[int] = None
    max_beam_size: Optional[int] = None
    beam_exact_ratio: float = 0.01
    max_iter: int = -1
    presort_indeg: bool = False


@dataclass
class Result:
    lower: int
    upper: int
    non_synchro: bool = False
    trace: list = field(default_factory=list)


def _arr(delta: Sequence[int]):
    return (ctypes.c_uint32 * len(delta))(*delta)


def default_upper_bound(n: int) -> int:
    """app/jit.hpp:152 — 1ULL * AUT_N * AUT_N * AUT_N / 6."""
    return n * n * n // 6


def exact(delta: Sequence[int], n: int, k: int, params: ExactParams = ExactParams(),
          lower: int = 0, upper: Optional[int] = None, trace_capacity: int = 0) -> Result:
    p = _ExactParams(int(params.dfs), int(params.dfs_shortcut), int(params.strict_memory_limit),
                     params.max_memory_mb, params.dfs_min_list_size,
                     params.bfs_small_list_size if params.bfs_small_list_size is not None else 16 * n,
                     params.threads)
    b = _Bounds(0, lower, default_upper_bound(n) if upper is None else upper)
    tr = None
    steps = None
    if trace_capacity:
        steps = (_TraceStep * trace_capacity)()
        tr = _Trace(steps, trace_capacity, 0)
    rc = lib().oracle_exact(_arr(delta), n, k, ctypes.byref(p), ctypes.byref(b),
                            ctypes.byref(tr) if tr is not None else None)
    if rc != 0:
        raise RuntimeError(f"oracle_exact failed with {rc}")
    out = Result(b.lower, b.upper, bool(b.non_synchro))
    if tr is not None:
        out.trace = [(steps[i].phase, steps[i].len, steps[i].list_bfs, steps[i].list_invbfs)
                     for i in range(tr.count)]
    return out


def beam(delta: Sequence[int], n: int, k: int, params: BeamParams = BeamParams(),
         lower: int = 0, upper: Optional[int] = None) -> Result:
    import math
    lg = math.log2(n)
    p = _BeamParams(int(params.beam_size if params.beam_size is not None else lg),
                    int(params.dynamic),
                    int(params.min_beam_size if params.min_beam_size is not None else n * lg),
                    int(params.max_beam_size if params.max_beam_size is not None else n * n * lg),
                    params.beam_exact_ratio, params.max_iter, int(params.presort_indeg))
    b = _Bounds(0, lower, default_upper_bound(n) if upper is None else upper)
    rc = lib().oracle_beam(_arr(delta), n, k, ctypes.byref(p), ctypes.byref(b))
    if rc != 0:
        raise RuntimeError(f"oracle_beam failed with {rc}")
    return Result(b.lower, b.upper, bool(b.non_synchro))


def brute(delta: Sequence[int], n: int, k: int) -> int:
    """Shortest reset length by exhaustive power-set BFS (n <= 24); -1 if none."""
    out = ctypes.c_int64()
    rc = lib().oracle_brute(_arr(delta), n, k, ctypes.byref(out))
    if rc != 0:
        raise RuntimeError(f"oracle_brute failed with {rc}")
    return out.value


def eppstein(delta: Sequence[int], n: int, k: int, lower: int = 0, upper: Optional[int] = None):
    """Eppstein's greedy upper bound: (Result, word) — word None when the bound is unchanged."""
    b = _Bounds(0, lower, default_upper_bound(n) if upper is None else upper)
    before = b.upper
    cap = n * n * n // 6 + n + 1
    buf = (ctypes.c_uint32 * cap)()
    wl = ctypes.c_uint64()
    rc = lib().oracle_eppstein(_arr(delta), n, k, ctypes.byref(b), buf, cap, ctypes.byref(wl))
    if rc != 0:
        raise RuntimeError(f"oracle_eppstein failed with {rc}")
    res = Result(b.lower, b.upper, bool(b.non_synchro))
    word = list(buf[:wl.value]) if (wl.value or b.upper != before) and not b.non_synchro else None
    return res, word


def apply_word(delta: Sequence[int], n: int, k: int, word: Sequence[int]) -> set:
    """Image of the full state set under `word` (the word check used by every test)."""
    cur = set(range(n))
    for a in word:
        cur = {delta[q * k + a] for q in cur}
    return cur
