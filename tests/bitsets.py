"""Test helpers: sets <-> the reference bitset layout (state q = bit q%64 of
word q/64, synchrolib/data_structures/subset.hpp:11-26) and plain-Python
restatements of the per-set operations the kernels perform."""
from __future__ import annotations

import numpy as np

MASK64 = (1 << 64) - 1


def words(n: int) -> int:
    return (n + 63) // 64


def to_rows(sets, n: int) -> np.ndarray:
    rw = words(n)
    out = np.zeros((len(sets), rw), dtype=np.uint64)
    for i, s in enumerate(sets):
        for q in s:
            out[i, q // 64] |= np.uint64(1 << (q % 64))
    return out


def from_rows(rows: np.ndarray, n: int):
    out = []
    for r in np.asarray(rows).reshape(-1, words(n)):
        s = set()
        for w, v in enumerate(r.tolist()):
            while v:
                b = (v & -v).bit_length() - 1
                s.add(64 * w + b)
                v &= v - 1
        out.append(frozenset(s))
    return out


def random_sets(rng: np.random.Generator, n: int, count: int, density: float):
    m = rng.random((count, n)) < density
    return [frozenset(np.nonzero(row)[0].tolist()) for row in m]


def image(delta, k, a, s):
    return frozenset(delta[q * k + a] for q in s)


def preimage(delta, n, k, a, s):
    return frozenset(q for q in range(n) if delta[q * k + a] in s)


def rev64(v: int) -> int:
    return int(f"{v:064b}"[::-1], 2)


def ref_order_key(row) -> tuple:
    """Subset::operator< (subset.hpp:71-77): compare bit-reversed words."""
    return tuple(rev64(int(x)) for x in row)


def brute_contains(S, C, proper: bool):
    """results[i] = exists s in S with s ⊆ C[i] (s != C[i] if proper)."""
    out = []
    for c in C:
        hit = any(s <= c and (not proper or s != c) for s in S)
        out.append(1 if hit else 0)
    return out
