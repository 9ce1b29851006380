"""Seeded automaton generators (host side).

The reference's generator (scripts/generate.py:19-53) draws random
transitions from numpy's ``default_rng``, whose stream is not pinned by the
reference.  Here every random automaton comes from SplitMix64 (Steele,
Lea & Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014)
with Lemire's multiply-shift range reduction, so the same seed gives the same
automaton on every machine and in every language that restates it.

Families:
  random      delta(q, a) uniform in [0, n)                 (generate.py:19-23)
  cerny       C_n: a: q -> q+1 mod n, b: 0 -> 1, others fixed; reset length (n-1)^2
  cerny_ref   the reference script's labelling of C_n       (generate.py:25-33)
  slowlysink  k = n-1, reset length n(n-1)/2                (generate.py:34-53)
  hard        Automaton::generate_hard                      (automaton.hpp:97-115)
"""
from __future__ import annotations

import argparse
from typing import Iterator, List, Tuple

MASK = (1 << 64) - 1


def splitmix64(seed: int) -> Iterator[int]:
    state = seed & MASK
    while True:
        state = (state + 0x9E3779B97F4A7C15) & MASK
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        yield z ^ (z >> 31)


def random_dfa(n: int, k: int, seed: int) -> List[int]:
    """delta[q*k + a], each uniform in [0, n) (multiply-shift of a 64-bit draw)."""
    g = splitmix64(seed)
    return [(next(g) * n) >> 64 for _ in range(n * k)]


def cerny(n: int) -> List[int]:
    """C_n with letter 0: q -> q+1 mod n, letter 1: 0 -> 1, other states fixed."""
    d = [0] * (2 * n)
    for q in range(n):
        d[2 * q] = (q + 1) % n
        d[2 * q + 1] = q
    if n > 1:
        d[1] = 1
    return d


def cerny_ref(n: int) -> List[int]:
    """The reference script's labelling of C_n (generate.py:25-33): letter 0 is
    the cycle q -> q+1, n-1 -> 0; letter 1 fixes every state but n-1 -> 0."""
    d = [0] * (2 * n)
    for i in range(n - 1):
        d[2 * i] = i + 1
        d[2 * i + 1] = i
    return d


def slowlysink(n: int) -> List[int]:
    """generate.py:34-53 (k = n - 1)."""
    k = n - 1
    d = [0] * (k * n)
    for a in range(n - 1):
        for q in range(1, n):
            d[q * k + a] = q
        d[a * k + a] = a + 1
        d[(a + 1) * k + a] = a
    d[0] = 0
    return d


def hard(n: int) -> List[int]:
    """Automaton::generate_hard (automaton.hpp:102-115), k = 2."""
    d = [0] * (2 * n)
    for i in range(n - 1):
        d[2 * i] = d[2 * i + 1] = i + 1
    d[2 * (n - 1)] = 0
    d[2 * (n - 1) + 1] = 1
    d[2 * 1 + 1] = 0
    d[2 * 0 + 1] = 3
    d[2 * 2 + 1] = 3
    return d


def batch(count: int, seed: int, n_range=(32, 160), k_choices=(2, 3)) -> List[Tuple[int, int, List[int]]]:
    """Uneven batch: n uniform in n_range (inclusive), k uniform in k_choices,
    instance i seeded with a draw of the master stream."""
    g = splitmix64(seed)
    out = []
    lo, hi = n_range
    for _ in range(count):
        n = lo + ((next(g) * (hi - lo + 1)) >> 64)
        k = k_choices[(next(g) * len(k_choices)) >> 64]
        s = next(g)
        out.append((n, k, random_dfa(n, k, s)))
    return out


def to_text(autos) -> str:
    """Reference input format (docs/install.md:42-50)."""
    return "".join(f"{k} {n}\n" + " ".join(map(str, d)) + "\n" for n, k, d in autos)


def main() -> None:
    ap = argparse.ArgumentParser(description="Generate automata in the reference input format")
    ap.add_argument("K", type=int)
    ap.add_argument("N", type=int)
    ap.add_argument("-o", "--output", required=True)
    ap.add_argument("-t", "--type", choices=["random", "cerny", "cerny_ref", "slowlysink", "hard"], default="random")
    ap.add_argument("-s", "--seed", type=int, default=1)
    ap.add_argument("-c", "--count", type=int, default=1)
    ap.add_argument("-a", "--append", action="store_true")
    a = ap.parse_args()
    autos = []
    for i in range(a.count):
        if a.type == "random":
            autos.append((a.N, a.K, random_dfa(a.N, a.K, a.seed + i)))
        elif a.type == "cerny":
            autos.append((a.N, 2, cerny(a.N)))
        elif a.type == "cerny_ref":
            autos.append((a.N, 2, cerny_ref(a.N)))
        elif a.type == "slowlysink":
            autos.append((a.N, a.N - 1, slowlysink(a.N)))
        else:
            autos.append((a.N, 2, hard(a.N)))
    with open(a.output, "a" if a.append else "w") as f:
        f.write(to_text(autos))


if __name__ == "__main__":
    main()
