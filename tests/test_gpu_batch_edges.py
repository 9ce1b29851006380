"""Edge cases of the persistent batched launch (k_small_batch) against the
oracle: one-letter and two-state automata, permutation automata (no reset
word), Černý automata whose searches are deep (up to 361 letters, and one
past the launch's 512-letter search bound), every set width 1..4 in one
batch, and automata whose layers outgrow the launch's capacities.  Each
batch is solved with the batched launch taking every automaton it accepts
(batched_limit 1024) and with the launch turned off (batched_limit -1):
both routes must give the oracle's bounds and verified words."""
import random

import pytest

import oracle
from synchrowords_gb300 import generate as gen

pytestmark = pytest.mark.gpu

PLAN = '{"algorithms": [{"name": "Exact", "config": {}}]}'


def permutation_automaton(n, k, rng):
    d = [0] * (n * k)
    for a in range(k):
        p = list(range(n))
        rng.shuffle(p)
        for q in range(n):
            d[q * k + a] = p[q]
    return d


def edge_batch():
    rng = random.Random(77)
    autos = []
    for n in (2, 3, 5, 9):  # one letter: synchronizing only if the map funnels into a fixed point
        for _ in range(3):
            autos.append((n, 1, [rng.randrange(n) for _ in range(n)]))
    for k in (1, 2, 3, 4):  # two states
        for _ in range(2):
            autos.append((2, k, [rng.randrange(2) for _ in range(2 * k)]))
    for n, k in ((6, 2), (20, 3), (70, 2)):  # permutations: no reset word
        autos.append((n, k, permutation_automaton(n, k, rng)))
    for n in (5, 12, 20, 24):  # Černý: (n-1)^2 = 16, 121, 361, 529 (past the 512 bound)
        autos.append((n, 2, gen.cerny(n)))
    for n, k, s in ((33, 2, 1), (64, 3, 2), (65, 2, 3), (100, 2, 4), (128, 2, 5), (129, 2, 6), (150, 2, 7),
                    (192, 2, 8), (193, 2, 9), (230, 2, 10), (256, 2, 12), (90, 4, 13)):
        autos.append((n, k, gen.random_dfa(n, k, 5000 + s)))
    return autos


def synchronizing(d, n, k):
    """Pair-graph check: every pair of states reaches the diagonal."""
    pre = [[[] for _ in range(k)] for _ in range(n)]
    for q in range(n):
        for a in range(k):
            pre[d[q * k + a]][a].append(q)
    seen = [[False] * n for _ in range(n)]
    todo = [(q, q) for q in range(n)]
    for q in range(n):
        seen[q][q] = True
    reached = n
    while todo:
        p, q = todo.pop()
        for a in range(k):
            for x in pre[p][a]:
                for y in pre[q][a]:
                    x1, y1 = min(x, y), max(x, y)
                    if not seen[x1][y1]:
                        seen[x1][y1] = True
                        reached += 1
                        todo.append((x1, y1))
    return reached == n * (n + 1) // 2


@pytest.fixture(scope="module")
def expected():
    """(has no reset word, lower, upper): the oracle's Exact lengths; the
    reference's Exact has no synchronisation test (it reports its upper bound
    for an automaton without a reset word), the library reports non_synchro."""
    out = []
    for n, k, d in edge_batch():
        if not synchronizing(d, n, k):
            out.append((True, None, None))
            continue
        r = oracle.exact(d, n, k)
        out.append((False, r.lower, r.upper))
    return out


@pytest.mark.parametrize("limit", [1024.0, -1.0])
def test_batched_launch_edges_match_oracle(native_lib, expected, limit):
    import synchrowords_gb300 as sw
    autos = edge_batch()
    with sw.Context(0) as ctx:
        ctx.set_batch_tuning(workers=4, batched_limit=limit)
        res = ctx.solve_batch(autos, PLAN)
    assert any(e[0] for e in expected) and not all(e[0] for e in expected)
    for i, ((n, k, d), r, (ns, lo, up)) in enumerate(zip(autos, res, expected)):
        assert r.non_synchro == ns, (i, n, k)
        if ns:
            continue
        assert (r.lower, r.upper) == (lo, up), (i, n, k, r.lower, r.upper, lo, up)
        assert r.word is not None and len(r.word) == up, (i, n, k)
        assert len(oracle.apply_word(d, n, k, r.word)) == 1, (i, n, k)
