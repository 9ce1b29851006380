"""synchrowords GB300: GPU exact shortest-reset-word search (SynchroLib drop-in).

Python front end over the C ABI in ``include/synchrowords.h``.  It mirrors the
reference's plugin interface (jit/jitmain.cpp:11-49): a plan (the reference's
config JSON) is evaluated for one automaton and its algorithms run in order on
the GPU, producing an ``AlgoResult``-like record (bounds, per-algorithm
milliseconds and, new here, a verified reset word).

The library has no CPU path: loading fails loudly when the compiled library
is missing, and creating a context fails when no CUDA device is present.
"""
from __future__ import annotations

import ctypes
import itertools
from dataclasses import dataclass, field
from pathlib import Path
from typing import List, Optional, Sequence, Tuple

import numpy as np

__all__ = ["Context", "Result", "SynchroError", "read_automata", "format_result", "plan_from_json",
           "eval_expression", "library_path", "load_library", "MAX_STATES", "MAX_LETTERS"]

PKG = Path(__file__).resolve().parent
MAX_STATES = 512
MAX_LETTERS = 16
NAME_LEN = 16
MAX_ALGOS = 16


def library_path() -> Path:
    return PKG / "_build" / "libsynchrowords.so"


class SynchroError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


# ---- ctypes mirrors of include/synchrowords.h --------------------------------
class _ExactCfg(ctypes.Structure):
    _fields_ = [("dfs", ctypes.c_int32), ("dfs_shortcut", ctypes.c_int32), ("strict_memory_limit", ctypes.c_int32),
                ("max_memory_mb", ctypes.c_uint64), ("dfs_min_list_size", ctypes.c_uint64),
                ("bfs_small_list_size", ctypes.c_uint64), ("reductions", ctypes.c_int32)]


class _BeamCfg(ctypes.Structure):
    _fields_ = [("beam_size", ctypes.c_uint64), ("dynamic", ctypes.c_int32), ("min_beam_size", ctypes.c_uint64),
                ("max_beam_size", ctypes.c_uint64), ("beam_exact_ratio", ctypes.c_double),
                ("max_iter", ctypes.c_int64), ("presort_indeg", ctypes.c_int32)]


class _BruteCfg(ctypes.Structure):
    _fields_ = [("max_n", ctypes.c_uint64)]


class _EppsteinCfg(ctypes.Structure):
    _fields_ = [("transition_tables", ctypes.c_int32), ("find_word", ctypes.c_int32)]


class _ReduceCfg(ctypes.Structure):
    _fields_ = [("min_n", ctypes.c_uint64), ("list_size_threshold", ctypes.c_uint64)]


class _LearnedBeamCfg(ctypes.Structure):
    _fields_ = [("beam_size", ctypes.c_uint64), ("max_iter", ctypes.c_int64), ("order", ctypes.c_int32)]


class _Algo(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("name", ctypes.c_char * NAME_LEN), ("exact", _ExactCfg),
                ("beam", _BeamCfg), ("brute", _BruteCfg), ("eppstein", _EppsteinCfg), ("reduce", _ReduceCfg),
                ("learned_beam", _LearnedBeamCfg)]


class _Plan(ctypes.Structure):
    _fields_ = [("upper_bound", ctypes.c_uint64), ("threads", ctypes.c_uint32), ("gpu", ctypes.c_int32),
                ("gpu_max_memory_mb", ctypes.c_uint64), ("n_algorithms", ctypes.c_uint32),
                ("algorithms", _Algo * MAX_ALGOS)]


class _Run(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * NAME_LEN), ("ms", ctypes.c_uint64)]


class _Stats(ctypes.Structure):
    _fields_ = [("subsets_expanded", ctypes.c_uint64), ("subsets_kept", ctypes.c_uint64),
                ("trie_queries", ctypes.c_uint64), ("logical_pairs", ctypes.c_uint64),
                ("meet_pairs", ctypes.c_uint64), ("bfs_steps", ctypes.c_uint64), ("ibfs_steps", ctypes.c_uint64),
                ("dfs_sets", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64), ("device_ms", ctypes.c_double), ("reduce_bfs_steps", ctypes.c_uint64),
                ("reduced_states", ctypes.c_uint64)]


class _Result(ctypes.Structure):
    _fields_ = [("non_synchro", ctypes.c_int32), ("mlsw_lower_bound", ctypes.c_uint64),
                ("mlsw_upper_bound", ctypes.c_uint64), ("has_word", ctypes.c_int32), ("word_len", ctypes.c_uint32),
                ("word", ctypes.POINTER(ctypes.c_uint32)), ("word_capacity", ctypes.c_uint32),
                ("n_runs", ctypes.c_uint32), ("runs", _Run * MAX_ALGOS), ("stats", _Stats)]


class _BatchTuning(ctypes.Structure):
    _fields_ = [("workers", ctypes.c_uint32), ("batched_limit", ctypes.c_double), ("cluster_size", ctypes.c_int32),
                ("cluster_limit", ctypes.c_double)]


DEFAULT_CLUSTER_LIMIT = 160.0  # the library's default (include/synchrowords.h)


class _BatchProfile(ctypes.Structure):
    _fields_ = [("small_solved", ctypes.c_uint32), ("cluster_solved", ctypes.c_uint32),
                ("streamed", ctypes.c_uint32), ("launches", ctypes.c_uint32), ("device_ms", ctypes.c_double),
                ("meet_pairs", ctypes.c_uint64), ("children", ctypes.c_uint64), ("staged_bytes", ctypes.c_uint64),
                ("steps", ctypes.c_uint64), ("graph_replays", ctypes.c_uint32)]


class _ScanShape(ctypes.Structure):
    _fields_ = [("tile_rows", ctypes.c_int32), ("warps", ctypes.c_int32), ("tiles_per_super", ctypes.c_int32),
                ("grid_factor", ctypes.c_int32)]


class _ScanTuned(ctypes.Structure):
    _fields_ = [("words", ctypes.c_uint32), ("size_class", ctypes.c_uint32), ("checks", ctypes.c_uint64),
                ("ms_start", ctypes.c_double), ("ms_best", ctypes.c_double), ("shape", _ScanShape)]


SCAN_SIZE_CLASSES = 2        # class 0: lists of fewer than SCAN_LARGE_ROWS rows; class 1: larger
SCAN_LARGE_ROWS = 32768
DEFAULT_SCAN_SHAPE = {"tile_rows": 64, "warps": 8, "tiles_per_super": 16, "grid_factor": 16}


class _KernelProfile(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_uint64), ("ms", ctypes.c_double), ("bytes", ctypes.c_double)]


PROFILE_CLASSES = ("subset_query", "expand", "radix_sort", "other")

_lib = None

_U32P = ctypes.POINTER(ctypes.c_uint32)
_U64P = ctypes.POINTER(ctypes.c_uint64)


def load_library():
    """Load the compiled library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        raise ImportError(f"synchrowords_gb300 native library not built ({path}); "
                          "run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(str(path))
    lib.sw_version.restype = ctypes.c_char_p
    lib.sw_last_error.restype = ctypes.c_char_p
    lib.sw_plan_from_json.argtypes = [ctypes.c_char_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(_Plan)]
    lib.sw_eval_expression.argtypes = [ctypes.c_char_p, ctypes.c_uint32, ctypes.c_uint32, _U64P,
                                       ctypes.POINTER(ctypes.c_double)]
    lib.sw_context_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    lib.sw_context_destroy.argtypes = [ctypes.c_void_p]
    lib.sw_solve.argtypes = [ctypes.c_void_p, _U32P, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(_Plan),
                             ctypes.POINTER(_Result)]
    lib.sw_solve_json.argtypes = [ctypes.c_void_p, _U32P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_char_p,
                                  ctypes.POINTER(_Result)]
    lib.sw_apply_transition.argtypes = [ctypes.c_void_p, _U32P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                        ctypes.c_int32, _U64P, _U64P, ctypes.c_uint64]
    lib.sw_subsets_check.argtypes = [ctypes.c_void_p, ctypes.c_uint32, _U64P, ctypes.c_uint64, _U64P,
                                     ctypes.c_uint64, ctypes.c_int32, ctypes.POINTER(ctypes.c_uint8)]
    lib.sw_sort_unique.argtypes = [ctypes.c_void_p, ctypes.c_uint32, _U64P, ctypes.c_uint64, _U64P]
    lib.sw_solve_batch.argtypes = [ctypes.c_void_p, ctypes.c_uint32, _U32P, _U32P, _U32P, ctypes.c_char_p,
                                   ctypes.POINTER(_Result), ctypes.c_uint32]
    _F64P = ctypes.POINTER(ctypes.c_double)
    lib.sw_autotune_batch.argtypes = [ctypes.c_void_p, ctypes.c_uint32, _U32P, _U32P, _U32P, ctypes.c_char_p,
                                      ctypes.POINTER(_Result), _U32P, ctypes.c_uint32, _F64P, ctypes.c_uint32,
                                      ctypes.c_uint32, _F64P, ctypes.POINTER(_BatchTuning)]
    lib.sw_get_batch_tuning.argtypes = [ctypes.c_void_p, ctypes.POINTER(_BatchTuning)]
    lib.sw_set_batch_tuning.argtypes = [ctypes.c_void_p, ctypes.POINTER(_BatchTuning)]
    lib.sw_batch_last_profile.argtypes = [ctypes.c_void_p, ctypes.POINTER(_BatchProfile)]
    lib.sw_autotune_cluster.argtypes = [ctypes.c_void_p, ctypes.c_uint32, _U32P, _U32P, _U32P, ctypes.c_char_p,
                                        ctypes.POINTER(_Result), ctypes.POINTER(ctypes.c_int32), ctypes.c_uint32,
                                        ctypes.POINTER(ctypes.c_double), ctypes.c_uint32, ctypes.c_uint32,
                                        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_BatchTuning)]
    lib.sw_get_scan_shape.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(_ScanShape)]
    lib.sw_set_scan_shape.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(_ScanShape)]
    lib.sw_scan_shape_check.argtypes = [ctypes.c_uint32, ctypes.POINTER(_ScanShape)]
    lib.sw_autotune_scan.argtypes = [ctypes.c_void_p, ctypes.c_uint32, _U32P, _U32P, _U32P, ctypes.c_char_p,
                                     ctypes.c_uint32, ctypes.POINTER(_ScanTuned), ctypes.c_uint32, _U32P]
    lib.sw_subsets_check_device_noalloc.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64,
                                                     ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32,
                                                     ctypes.c_void_p, ctypes.c_void_p]
    _F32P = ctypes.POINTER(ctypes.c_float)
    lib.sw_context_set_model.argtypes = [ctypes.c_void_p, _F32P, ctypes.c_uint32]
    lib.sw_context_get_model.argtypes = [ctypes.c_void_p, _F32P, ctypes.c_uint32]
    lib.sw_state_features.argtypes = [_U32P, ctypes.c_uint32, ctypes.c_uint32, _F32P]
    lib.sw_distance_pairs.argtypes = [ctypes.c_void_p, _U32P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                      ctypes.c_uint64, _U64P, _F32P, _U32P, ctypes.c_uint64, _U64P, _U32P]
    lib.sw_mlp_forward.argtypes = [ctypes.c_void_p, _F32P, _U32P, ctypes.c_uint32, ctypes.c_uint32, _U64P,
                                   ctypes.c_uint64, _F32P]
    lib.sw_mlp_gradient.argtypes = [ctypes.c_void_p, _F32P, _U32P, ctypes.c_uint32, ctypes.c_uint32, _U64P, _F32P,
                                    ctypes.c_uint64, _F32P, _F32P]
    lib.sw_mlp_train_ranked.argtypes = [ctypes.c_void_p, _F32P, ctypes.c_uint32, _U32P, _U32P, _U32P, _U64P, _U64P,
                                        _F32P, _U32P, ctypes.c_float, ctypes.c_uint32, ctypes.c_uint32,
                                        ctypes.c_float, ctypes.c_uint64, ctypes.POINTER(ctypes.c_float)]
    lib.sw_mlp_train.argtypes = [ctypes.c_void_p, _F32P, ctypes.c_uint32, _U32P, _U32P, _U32P, _U64P, _U64P, _F32P,
                                 ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, ctypes.c_uint64, _F32P]
    lib.sw_profile_begin.argtypes = [ctypes.c_void_p]
    lib.sw_profile_end.argtypes = [ctypes.c_void_p, ctypes.POINTER(_KernelProfile)]
    lib.sw_context_stream.argtypes = [ctypes.c_void_p]
    lib.sw_context_stream.restype = ctypes.c_void_p
    _lib = lib
    return lib


def _check(rc: int) -> None:
    if rc != 0:
        raise SynchroError(rc, load_library().sw_last_error().decode())


def _u32(a: Sequence[int]) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32))


def eval_expression(expr: str, n: int, k: int) -> Tuple[int, float]:
    """(uint64 value, double value) of a config expression with AUT_N = n, AUT_K = k."""
    u = ctypes.c_uint64()
    d = ctypes.c_double()
    _check(load_library().sw_eval_expression(expr.encode(), n, k, ctypes.byref(u), ctypes.byref(d)))
    return u.value, d.value


def check_scan_shape(words: int, tile_rows: int = 64, warps: int = 8, tiles_per_super: int = 16,
                     grid_factor: int = 16) -> None:
    """Raise SynchroError unless this is a valid subset-check launch shape for
    rows of `words` 64-bit words (host-only; needs no device)."""
    s = _ScanShape(tile_rows, warps, tiles_per_super, grid_factor)
    _check(load_library().sw_scan_shape_check(words, ctypes.byref(s)))


def plan_from_json(text: str, n: int, k: int) -> dict:
    """Evaluated plan as a dict (the library's view of the reference config)."""
    p = _Plan()
    _check(load_library().sw_plan_from_json(text.encode(), n, k, ctypes.byref(p)))
    algos = []
    for i in range(p.n_algorithms):
        a = p.algorithms[i]
        d = {"kind": a.kind, "name": a.name.decode()}
        if a.kind == 1:
            d.update({f: getattr(a.exact, f) for f, _ in _ExactCfg._fields_})
        elif a.kind == 2:
            d.update({f: getattr(a.beam, f) for f, _ in _BeamCfg._fields_})
        elif a.kind == 3:
            d.update({f: getattr(a.brute, f) for f, _ in _BruteCfg._fields_})
        elif a.kind == 4:
            d.update({f: getattr(a.eppstein, f) for f, _ in _EppsteinCfg._fields_})
        elif a.kind == 5:
            d.update({f: getattr(a.reduce, f) for f, _ in _ReduceCfg._fields_})
        elif a.kind == 6:
            d.update({f: getattr(a.learned_beam, f) for f, _ in _LearnedBeamCfg._fields_})
        algos.append(d)
    return {"upper_bound": p.upper_bound, "threads": p.threads, "gpu": p.gpu,
            "gpu_max_memory_mb": p.gpu_max_memory_mb, "algorithms": algos}


@dataclass
class Result:
    """AlgoResult (synchrolib/algorithm/algorithm.hpp:19-42) plus statistics."""
    non_synchro: bool
    lower: int
    upper: int
    word: Optional[List[int]]
    runs: List[Tuple[str, int]]
    stats: dict = field(default_factory=dict)


MLP_PARAMS = 26049
STATE_FEATURES = 16
DEFAULT_MODEL = Path(__file__).resolve().parent / "models" / "distance_mlp.f32"
_F32 = ctypes.POINTER(ctypes.c_float)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def load_model(path=DEFAULT_MODEL) -> np.ndarray:
    """Parameters of the learned distance model (MLP_PARAMS little-endian float32)."""
    p = np.fromfile(str(path), dtype="<f4")
    if p.size != MLP_PARAMS:
        raise ValueError(f"{path}: expected {MLP_PARAMS} floats, found {p.size}")
    return p.astype(np.float32)


def state_features(delta: Sequence[int], n: int, k: int) -> np.ndarray:
    out = np.zeros((n, STATE_FEATURES), dtype=np.float32)
    _check(load_library().sw_state_features(_u32(delta).ctypes.data_as(_U32P), n, k, out.ctypes.data_as(_F32)))
    return out


class Context:
    """One CUDA device with persistent buffers (not thread-safe).

    The packaged distance model (models/distance_mlp.f32), when present, is
    loaded so that plans with a LearnedBeam entry run as they are."""

    def __init__(self, device: int = 0, model=DEFAULT_MODEL):
        self._lib = load_library()
        self._h = ctypes.c_void_p()
        _check(self._lib.sw_context_create(device, ctypes.byref(self._h)))
        if model is not None and Path(model).exists():
            self.set_model(load_model(model))

    def set_model(self, params) -> None:
        p = _f32(params)
        _check(self._lib.sw_context_set_model(self._h, p.ctypes.data_as(_F32), p.size))

    def get_model(self) -> np.ndarray:
        p = np.zeros(MLP_PARAMS, dtype=np.float32)
        _check(self._lib.sw_context_get_model(self._h, p.ctypes.data_as(_F32), MLP_PARAMS))
        return p

    def distance_pairs(self, delta, n: int, k: int, per_layer: int = 256, max_inverse_sets: int = 4_000_000,
                       capacity: int = 1 << 20):
        """(sets [count, 8] uint64 in the reference layout, labels float32,
        forward depths uint32, reset length)."""
        sets = np.zeros((capacity, 8), dtype=np.uint64)
        labels = np.zeros(capacity, dtype=np.float32)
        depths = np.zeros(capacity, dtype=np.uint32)
        cnt, length = ctypes.c_uint64(), ctypes.c_uint32()
        _check(self._lib.sw_distance_pairs(self._h, _u32(delta).ctypes.data_as(_U32P), n, k, per_layer,
                                           max_inverse_sets, sets.ctypes.data_as(_U64P), labels.ctypes.data_as(_F32),
                                           depths.ctypes.data_as(_U32P), capacity, ctypes.byref(cnt),
                                           ctypes.byref(length)))
        c = cnt.value
        return sets[:c].copy(), labels[:c].copy(), depths[:c].copy(), length.value

    def mlp_forward(self, params, delta, n: int, k: int, sets: np.ndarray) -> np.ndarray:
        s = np.ascontiguousarray(sets, dtype=np.uint64).reshape(-1, 8)
        out = np.zeros(len(s), dtype=np.float32)
        p = _f32(params)
        _check(self._lib.sw_mlp_forward(self._h, p.ctypes.data_as(_F32), _u32(delta).ctypes.data_as(_U32P), n, k,
                                        s.ctypes.data_as(_U64P), len(s), out.ctypes.data_as(_F32)))
        return out

    def mlp_gradient(self, params, delta, n: int, k: int, sets: np.ndarray, labels) -> Tuple[np.ndarray, float]:
        s = np.ascontiguousarray(sets, dtype=np.uint64).reshape(-1, 8)
        t = _f32(labels)
        g = np.zeros(MLP_PARAMS, dtype=np.float32)
        loss = ctypes.c_float()
        p = _f32(params)
        _check(self._lib.sw_mlp_gradient(self._h, p.ctypes.data_as(_F32), _u32(delta).ctypes.data_as(_U32P), n, k,
                                         s.ctypes.data_as(_U64P), t.ctypes.data_as(_F32), len(s),
                                         g.ctypes.data_as(_F32), ctypes.byref(loss)))
        return g, loss.value

    def mlp_train(self, params, automata, sets_per_automaton, labels_per_automaton, epochs: int = 1,
                  batch: int = 512, lr: float = 1e-3, seed: int = 1, groups_per_automaton=None,
                  rank_weight: float = 0.0) -> Tuple[np.ndarray, float]:
        """Adam training; returns (trained parameters, mean batch loss of the last epoch).  With
        groups (one id per set, e.g. its BFS layer) and rank_weight > 0 the loss adds a pairwise
        ranking term within each group."""
        p = _f32(params).copy()
        deltas = np.concatenate([_u32(d) for _, _, d in automata])
        ns = _u32([n for n, _, _ in automata])
        ks = _u32([k for _, k, _ in automata])
        offs = np.zeros(len(automata) + 1, dtype=np.uint64)
        offs[1:] = np.cumsum([len(l) for l in labels_per_automaton])
        sets = np.ascontiguousarray(np.concatenate([np.asarray(s, dtype=np.uint64).reshape(-1, 8)
                                                    for s in sets_per_automaton]), dtype=np.uint64)
        labels = _f32(np.concatenate(labels_per_automaton))
        loss = ctypes.c_float()
        grp = _u32(np.concatenate(groups_per_automaton)) if groups_per_automaton is not None else None
        _check(self._lib.sw_mlp_train_ranked(
            self._h, p.ctypes.data_as(_F32), len(automata), deltas.ctypes.data_as(_U32P), ns.ctypes.data_as(_U32P),
            ks.ctypes.data_as(_U32P), offs.ctypes.data_as(_U64P), sets.ctypes.data_as(_U64P),
            labels.ctypes.data_as(_F32), grp.ctypes.data_as(_U32P) if grp is not None else None,
            rank_weight if grp is not None else 0.0, epochs, batch, lr, seed, ctypes.byref(loss)))
        return p, loss.value

    def close(self) -> None:
        if self._h:
            self._lib.sw_context_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, delta: Sequence[int], n: int, k: int, plan_json: str) -> Result:
        d = _u32(delta)
        if d.size != n * k:
            raise ValueError("delta must have n*k entries")
        cap = max(1 << 16, 4 * n * n)
        buf = np.zeros(cap, dtype=np.uint32)
        r = _Result()
        r.word = buf.ctypes.data_as(_U32P)
        r.word_capacity = cap
        _check(self._lib.sw_solve_json(self._h, d.ctypes.data_as(_U32P), n, k, plan_json.encode(), ctypes.byref(r)))
        word = buf[: r.word_len].tolist() if r.has_word else None
        runs = [(r.runs[i].name.decode(), r.runs[i].ms) for i in range(r.n_runs)]
        stats = {f: getattr(r.stats, f) for f, _ in _Stats._fields_}
        return Result(bool(r.non_synchro), r.mlsw_lower_bound, r.mlsw_upper_bound, word, runs, stats)

    @staticmethod
    def _batch_buffers(automata):
        count = len(automata)
        ns = np.fromiter((a[0] for a in automata), dtype=np.uint32, count=count)
        ks = np.fromiter((a[1] for a in automata), dtype=np.uint32, count=count)
        total = int(np.dot(ns.astype(np.int64), ks.astype(np.int64)))
        if any(len(a[2]) != a[0] * a[1] for a in automata):
            raise ValueError("each automaton needs n * k transitions")
        deltas = np.fromiter(itertools.chain.from_iterable(a[2] for a in automata), dtype=np.uint32, count=total)
        # one word buffer for the batch: automaton i gets max(4096, 4 n^2) entries
        caps = np.maximum(1 << 12, 4 * ns.astype(np.uint64) ** 2)
        offs = np.zeros(count + 1, dtype=np.uint64)
        np.cumsum(caps, out=offs[1:])
        words = np.zeros(int(offs[-1]), dtype=np.uint32)
        res = (_Result * count)()
        raw = np.frombuffer(res, dtype=np.uint8).reshape(count, ctypes.sizeof(_Result))
        o = _Result.word.offset
        raw[:, o:o + 8] = (np.uint64(words.ctypes.data) + np.uint64(4) * offs[:-1]).view(np.uint8).reshape(count, 8)
        o = _Result.word_capacity.offset
        raw[:, o:o + 4] = caps.astype(np.uint32).view(np.uint8).reshape(count, 4)
        return ns, ks, deltas, res, words, offs

    @staticmethod
    def _batch_results(res, words, offs) -> List[Result]:
        out = []
        for i in range(len(res)):
            r = res[i]
            word = words[int(offs[i]): int(offs[i]) + r.word_len].tolist() if r.has_word else None
            runs = [(r.runs[j].name.decode(), r.runs[j].ms) for j in range(r.n_runs)]
            stats = {f: getattr(r.stats, f) for f, _ in _Stats._fields_}
            out.append(Result(bool(r.non_synchro), r.mlsw_lower_bound, r.mlsw_upper_bound, word, runs, stats))
        return out

    def solve_batch(self, automata: Sequence[Tuple[int, int, Sequence[int]]], plan_json: str,
                    workers: int = 0) -> List[Result]:
        """Solve many automata: plain-Exact automata of up to 256 states are
        searched on the device (a shared-memory persistent launch for the
        smallest, a thread-block-cluster launch for the rest), everything else
        and what those launches cannot finish on concurrent worker streams
        (workers = 0: the autotuned count, else min(count, 16))."""
        if len(automata) == 0:
            return []
        ns, ks, deltas, res, words, offs = self._batch_buffers(automata)
        _check(self._lib.sw_solve_batch(self._h, len(automata), deltas.ctypes.data_as(_U32P),
                                        ns.ctypes.data_as(_U32P), ks.ctypes.data_as(_U32P), plan_json.encode(),
                                        res, workers))
        return self._batch_results(res, words, offs)

    def autotune_batch(self, automata: Sequence[Tuple[int, int, Sequence[int]]], plan_json: str,
                       workers: Optional[Sequence[int]] = None, limits: Optional[Sequence[float]] = None,
                       reps: int = 1) -> dict:
        """Time the batch at each candidate worker count, then at each candidate
        batched-launch limit (n * log2 k), and keep the fastest as this context's
        tuning.  Returns {"workers", "batched_limit", "ms": {"workers": {w: ms},
        "batched_limit": {limit: ms}}}."""
        if len(automata) == 0:
            raise ValueError("empty batch")
        ns, ks, deltas, res, words, offs = self._batch_buffers(automata)
        wc = _u32(workers if workers is not None else (8, 12, 16, 24))
        lc = np.ascontiguousarray(np.asarray(limits if limits is not None else (-1.0, 104.0, 1024.0),
                                             dtype=np.float64))
        ms = np.zeros(len(wc) + len(lc), dtype=np.float64)
        best = _BatchTuning()
        f64 = ctypes.POINTER(ctypes.c_double)
        _check(self._lib.sw_autotune_batch(self._h, len(automata), deltas.ctypes.data_as(_U32P),
                                           ns.ctypes.data_as(_U32P), ks.ctypes.data_as(_U32P), plan_json.encode(),
                                           res, wc.ctypes.data_as(_U32P), len(wc), lc.ctypes.data_as(f64), len(lc),
                                           reps, ms.ctypes.data_as(f64), ctypes.byref(best)))
        return {"workers": int(best.workers), "batched_limit": float(best.batched_limit),
                "cluster_size": int(best.cluster_size), "cluster_limit": float(best.cluster_limit),
                "ms": {"workers": {int(w): float(t) for w, t in zip(wc, ms[:len(wc)])},
                       "batched_limit": {float(x): float(t) for x, t in zip(lc, ms[len(wc):])}}}

    def autotune_cluster(self, automata: Sequence[Tuple[int, int, Sequence[int]]], plan_json: str,
                         sizes: Optional[Sequence[int]] = None, limits: Optional[Sequence[float]] = None,
                         reps: int = 1) -> dict:
        """Time the batch at each candidate cluster size (CTAs per automaton of
        the cluster launch), then at each candidate cluster limit (n * log2 k
        of the automata it takes), and keep the fastest as this context's
        tuning.  Returns the tuning plus {"ms": {"cluster_size": {s: ms},
        "cluster_limit": {limit: ms}}}."""
        if len(automata) == 0:
            raise ValueError("empty batch")
        ns, ks, deltas, res, words, offs = self._batch_buffers(automata)
        sc = np.ascontiguousarray(np.asarray(sizes if sizes is not None else (2, 4, 8, 16), dtype=np.int32))
        lc = np.ascontiguousarray(np.asarray(limits if limits is not None else (-1.0, 128.0, 160.0, 200.0),
                                             dtype=np.float64))
        ms = np.zeros(len(sc) + len(lc), dtype=np.float64)
        best = _BatchTuning()
        f64 = ctypes.POINTER(ctypes.c_double)
        _check(self._lib.sw_autotune_cluster(self._h, len(automata), deltas.ctypes.data_as(_U32P),
                                             ns.ctypes.data_as(_U32P), ks.ctypes.data_as(_U32P), plan_json.encode(),
                                             res, sc.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), len(sc),
                                             lc.ctypes.data_as(f64), len(lc), reps, ms.ctypes.data_as(f64),
                                             ctypes.byref(best)))
        return {"workers": int(best.workers), "batched_limit": float(best.batched_limit),
                "cluster_size": int(best.cluster_size), "cluster_limit": float(best.cluster_limit),
                "ms": {"cluster_size": {int(s): float(t) for s, t in zip(sc, ms[:len(sc)])},
                       "cluster_limit": {float(x): float(t) for x, t in zip(lc, ms[len(sc):])}}}

    def get_scan_shape(self, words: int, size_class: int) -> dict:
        """Launch shape of the subset check for rows of `words` 64-bit words
        (1..8) and lists of size class 0 (< SCAN_LARGE_ROWS rows) or 1."""
        s = _ScanShape()
        _check(self._lib.sw_get_scan_shape(self._h, words, size_class, ctypes.byref(s)))
        return {f: int(getattr(s, f)) for f, _ in _ScanShape._fields_}

    def set_scan_shape(self, words: int, size_class: int, tile_rows: int = 64, warps: int = 8,
                       tiles_per_super: int = 16, grid_factor: int = 16) -> None:
        """tile_rows 32/64/128, warps 4/8/16, tiles_per_super 4/8/16/32,
        grid_factor 1..64; results never depend on the shape."""
        s = _ScanShape(tile_rows, warps, tiles_per_super, grid_factor)
        _check(self._lib.sw_set_scan_shape(self._h, words, size_class, ctypes.byref(s)))

    def autotune_scan(self, automata: Sequence[Tuple[int, int, Sequence[int]]], plan_json: Optional[str] = None,
                      reps: int = 1) -> list:
        """Tune the subset check's launch shape per (words, size class) on the
        checks these automata's solves make (coordinate descent over tile rows,
        warps, tiles per super-tile and grid factor, on CUDA-event time); the
        chosen shapes stay on this context.  One dict per key used: words,
        size_class, checks, ms_start, ms_best, shape."""
        if len(automata) == 0:
            raise ValueError("empty batch")
        ns, ks, deltas, _, _, _ = self._batch_buffers(automata)
        out = (_ScanTuned * 16)()
        cnt = ctypes.c_uint32(0)
        _check(self._lib.sw_autotune_scan(self._h, len(automata), deltas.ctypes.data_as(_U32P),
                                          ns.ctypes.data_as(_U32P), ks.ctypes.data_as(_U32P),
                                          plan_json.encode() if plan_json else None, reps, out, 16,
                                          ctypes.byref(cnt)))
        return [{"words": int(o.words), "size_class": int(o.size_class), "checks": int(o.checks),
                 "ms_start": float(o.ms_start), "ms_best": float(o.ms_best),
                 "shape": {f: int(getattr(o.shape, f)) for f, _ in _ScanShape._fields_}}
                for o in out[:min(cnt.value, 16)]]

    def get_batch_tuning(self) -> dict:
        t = _BatchTuning()
        _check(self._lib.sw_get_batch_tuning(self._h, ctypes.byref(t)))
        return {"workers": int(t.workers), "batched_limit": float(t.batched_limit),
                "cluster_size": int(t.cluster_size), "cluster_limit": float(t.cluster_limit)}

    def set_batch_tuning(self, workers: int = 0, batched_limit: float = 104.0, cluster_size: int = 0,
                         cluster_limit: float = DEFAULT_CLUSTER_LIMIT) -> None:
        """cluster_size: CTAs per automaton of the cluster launch (1..16, 0 = 8, -1 = off);
        cluster_limit: the largest n * log2(k) the cluster launch takes."""
        t = _BatchTuning(workers, batched_limit, cluster_size, cluster_limit)
        _check(self._lib.sw_set_batch_tuning(self._h, ctypes.byref(t)))

    def last_batch_profile(self) -> dict:
        """What the last solve_batch did on the device: automata per route,
        batched launches and their CUDA-event milliseconds, and the cluster
        launches' meet-check pairs, children, staged bytes and levels."""
        p = _BatchProfile()
        _check(self._lib.sw_batch_last_profile(self._h, ctypes.byref(p)))
        return {f: getattr(p, f) for f, _ in _BatchProfile._fields_}

    @property
    def stream(self) -> int:
        """cudaStream_t (as an integer) that every kernel of this context uses."""
        return int(self._lib.sw_context_stream(self._h) or 0)

    def profile_begin(self) -> None:
        _check(self._lib.sw_profile_begin(self._h))

    def profile_end(self) -> dict:
        """Per kernel class: launches, device ms (CUDA events) and algorithmic bytes."""
        arr = (_KernelProfile * len(PROFILE_CLASSES))()
        _check(self._lib.sw_profile_end(self._h, arr))
        return {name: {"launches": arr[i].launches, "ms": arr[i].ms, "bytes": arr[i].bytes}
                for i, name in enumerate(PROFILE_CLASSES)}

    # ---- kernel-level entry points (reference bitset layout) ----
    def apply_transition(self, delta, n: int, k: int, letter: int, inverse: bool, sets: np.ndarray) -> np.ndarray:
        d = _u32(delta)
        s = np.ascontiguousarray(sets, dtype=np.uint64)
        out = np.zeros_like(s)
        cnt = s.shape[0] if s.ndim > 1 else (s.size // max(1, (n + 63) // 64))
        _check(self._lib.sw_apply_transition(self._h, d.ctypes.data_as(_U32P), n, k, letter, int(inverse),
                                             s.ctypes.data_as(_U64P), out.ctypes.data_as(_U64P), cnt))
        return out

    def subsets_check(self, n: int, sets: np.ndarray, checks: np.ndarray, proper: bool = False) -> np.ndarray:
        s = np.ascontiguousarray(sets, dtype=np.uint64)
        c = np.ascontiguousarray(checks, dtype=np.uint64)
        rw = (n + 63) // 64
        ns, nc = s.size // rw, c.size // rw
        out = np.zeros(nc, dtype=np.uint8)
        _check(self._lib.sw_subsets_check(self._h, n, s.ctypes.data_as(_U64P), ns, c.ctypes.data_as(_U64P), nc,
                                          int(proper), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
        return out

    def sort_unique(self, n: int, sets: np.ndarray) -> np.ndarray:
        rw = (n + 63) // 64
        s = np.ascontiguousarray(sets, dtype=np.uint64).copy()
        cnt = ctypes.c_uint64()
        _check(self._lib.sw_sort_unique(self._h, n, s.ctypes.data_as(_U64P), s.size // rw, ctypes.byref(cnt)))
        return s.reshape(-1, rw)[: cnt.value]


def read_automata(path) -> List[Tuple[int, int, List[int]]]:
    """Automata in the reference's input format (app/io.hpp:136-159): "K N" then N*K ints."""
    toks = Path(path).read_text().split()
    out = []
    i = 0
    while i + 1 < len(toks):
        k, n = int(toks[i]), int(toks[i + 1])
        i += 2
        if n <= 0 or k <= 0:
            raise ValueError("N and K must be greater than 0")
        d = [int(x) for x in toks[i:i + n * k]]
        if len(d) != n * k:
            raise ValueError(f"Expected {n * k} integers, found {len(d)}")
        if any(x < 0 or x >= n for x in d):
            raise ValueError(f"Expected integer in range [0, {n - 1}]")
        i += n * k
        out.append((n, k, d))
    return out


def format_result(index: int, r: Result) -> str:
    """Output line of app/io.hpp:176-224: `ID: [lb, ub] ((Algo, ms), ...) {w...}`."""
    if r.non_synchro:
        return f"{index}: NON SYNCHRO"
    runs = ", ".join(f"({n}, {ms})" for n, ms in r.runs)
    s = f"{index}: [{r.lower}, {r.upper}] ({runs})"
    if r.word is not None:
        s += " {" + " ".join(map(str, r.word)) + "}"
    return s
