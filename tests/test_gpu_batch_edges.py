"""Edge cases of the persistent batched launch (k_small_batch) against the
compiled reference's answers (tests/golden/batch_edges.json): one-letter and
two-state automata, permutation automata (no reset word), Černý automata
whose searches are deep (up to 361 letters, and one past the launch's
512-letter search bound), every set width 1..4 in one batch, and automata
whose layers outgrow the launch's capacities.  Each batch is solved with the
batched launch taking every automaton it accepts (batched_limit 1024) and
with the launch turned off (batched_limit -1), each with the cluster launch
(k_cluster_batch: clusters of 8 or 2 CTAs) on or off: every route must give
the reference's lengths and verified words.  The reference's Exact has no
synchronisation test (it reports its upper bound for an automaton without a
reset word); the library reports non_synchro there, checked against a
pair-graph BFS."""
import json
from pathlib import Path

import pytest

import oracle

pytestmark = pytest.mark.gpu

GOLD = json.loads((Path(__file__).resolve().parent / "golden" / "batch_edges.json").read_text())
PLAN = json.dumps(GOLD["plan"])


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


@pytest.mark.parametrize("limit,cluster", [(1024.0, -1), (-1.0, -1), (-1.0, 0), (1024.0, 0), (-1.0, 2)])
def test_batched_launch_edges_match_reference(native_lib, limit, cluster):
    import synchrowords_gb300 as sw
    autos = [(c["n"], c["k"], c["delta"]) for c in GOLD["cases"]]
    sync = [synchronizing(d, n, k) for n, k, d in autos]
    assert any(sync) and not all(sync)
    with sw.Context(0) as ctx:
        ctx.set_batch_tuning(workers=4, batched_limit=limit, cluster_size=cluster)
        res = ctx.solve_batch(autos, PLAN)
    for i, ((n, k, d), r, s, c) in enumerate(zip(autos, res, sync, GOLD["cases"])):
        assert r.non_synchro == (not s), (i, n, k)
        if not s:
            continue
        want = c["reference"]
        assert (r.lower, r.upper) == (want["lower"], want["upper"]), (i, n, k, r.lower, r.upper, want)
        assert r.word is not None and len(r.word) == want["upper"], (i, n, k)
        assert len(oracle.apply_word(d, n, k, r.word)) == 1, (i, n, k)
