"""Kernel parity through the C ABI: layer expansion, subset check, sort-unique.

Bit-exact against plain-Python restatements of the reference operations
(PreprocessedTransition::apply, SubsetsImplicitTrie check, sort_keep_unique).
"""
import numpy as np
import pytest

from bitsets import (brute_contains, from_rows, image, preimage, random_sets, ref_order_key, to_rows, words)
from synchrowords_gb300.generate import random_dfa

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 5, 31, 32, 33, 48, 63, 64, 65, 100, 127, 128, 129, 200, 255, 256, 257, 320, 384, 448, 511, 512]


@pytest.mark.parametrize("n", SIZES)
def test_apply_transition_matches_definition(ctx, n):
    rng = np.random.default_rng(n)
    k = 3
    delta = random_dfa(n, k, 1000 + n)
    sets = [frozenset(), frozenset(range(n))]
    for dens in (0.02, 0.1, 0.5, 0.9):
        sets += random_sets(rng, n, 40, dens)
    rows = to_rows(sets, n)
    for a in range(k):
        fwd = from_rows(ctx.apply_transition(delta, n, k, a, False, rows), n)
        inv = from_rows(ctx.apply_transition(delta, n, k, a, True, rows), n)
        assert fwd == [image(delta, k, a, s) for s in sets]
        assert inv == [preimage(delta, n, k, a, s) for s in sets]


def test_apply_transition_empty_input(ctx):
    out = ctx.apply_transition([0, 1, 1, 0], 2, 2, 0, False, np.zeros((0, 1), dtype=np.uint64))
    assert out.size == 0


@pytest.mark.parametrize("n", [1, 7, 48, 64, 65, 128, 200, 256, 320, 384, 512])
@pytest.mark.parametrize("proper", [False, True])
def test_subsets_check_matches_brute_force(ctx, n, proper):
    rng = np.random.default_rng(7 * n + proper)
    S = random_sets(rng, n, 300, 0.08) + random_sets(rng, n, 50, 0.3)
    C = random_sets(rng, n, 400, 0.7) + random_sets(rng, n, 100, 0.95)
    # equal sets and duplicates exercise the proper / non-proper boundary
    C += S[:40]
    S += S[:10]
    C += [frozenset(range(n)), frozenset()]
    got = ctx.subsets_check(n, to_rows(S, n), to_rows(C, n), proper=proper).tolist()
    assert got == brute_contains(S, C, proper)


@pytest.mark.parametrize("m", [0, 1, 2, 3, 9, 17, 100, 2047, 2048, 2049, 5000, 40000])
def test_subsets_check_sizes(ctx, m):
    n = 96
    rng = np.random.default_rng(m)
    S = random_sets(rng, n, m, 0.05)
    C = random_sets(rng, n, 300, 0.8) + S[: min(m, 20)]
    got = ctx.subsets_check(n, to_rows(S, n), to_rows(C, n)).tolist()
    assert got == brute_contains(S, C, False)


def test_subsets_check_deep_chain(ctx):
    # nested sets {0..i}: the radix tree degenerates to a chain (stack fallback)
    n = 512
    S = [frozenset(range(i + 1)) for i in range(0, n, 3)]
    C = [frozenset(range(j)) for j in range(0, n + 1, 7)] + [frozenset(range(n)) - {0}]
    for proper in (False, True):
        got = ctx.subsets_check(n, to_rows(S, n), to_rows(C, n), proper=proper).tolist()
        assert got == brute_contains(S, C, proper)


@pytest.mark.parametrize("n", [3, 64, 65, 200, 384, 512])
@pytest.mark.parametrize("count", [0, 1, 5, 1000, 2048, 2049, 30000])
def test_sort_unique_reference_order(ctx, n, count):
    rng = np.random.default_rng(n * 31 + count)
    sets = random_sets(rng, n, count, 0.3)
    if count > 4:
        sets += sets[: count // 4]  # duplicates
    rows = to_rows(sets, n)
    got = ctx.sort_unique(n, rows)
    uniq = sorted({tuple(r.tolist()) for r in rows}, key=ref_order_key)
    assert [tuple(r.tolist()) for r in got] == uniq
