"""Exact / Beam parity on the GPU against the oracle (the CPU restatement of the
reference, itself pinned to the compiled reference) and word verification."""
import json
from pathlib import Path

import pytest

import oracle
from synchrowords_gb300.generate import cerny, hard, random_dfa, slowlysink

pytestmark = pytest.mark.gpu

EXACT = json.dumps({"algorithms": [{"name": "Exact", "config": {}}]})
BEAM_EXACT = json.dumps({
    "upper_bound": "1ULL * (AUT_N - 1) * (AUT_N - 1) + 1",
    "algorithms": [
        {"name": "Beam", "config": {"presort": "indeg", "dynamic": True,
                                    "min_beam_size": "AUT_N * std::log2(AUT_N)",
                                    "max_beam_size": "AUT_N * AUT_N * std::log2(AUT_N)",
                                    "beam_exact_ratio": 0.01}},
        {"name": "Exact", "config": {"dfs_min_list_size": "8192", "bfs_small_list_size": "AUT_N * AUT_K",
                                     "max_memory_mb": "12 * 1024"}}]})


def check_word(d, n, k, r):
    assert r.word is not None, "no word returned"
    assert len(r.word) == r.upper
    assert all(0 <= a < k for a in r.word)
    assert len(oracle.apply_word(d, n, k, r.word)) == 1


@pytest.mark.parametrize("seed", range(1, 17))
def test_random_n48_exact(ctx, seed):
    n, k = 48, 2
    d = random_dfa(n, k, seed)
    r = ctx.solve(d, n, k, EXACT)
    ref = oracle.exact(d, n, k)
    assert (r.lower, r.upper) == (ref.lower, ref.upper)
    check_word(d, n, k, r)


@pytest.mark.parametrize("n", [2, 3, 4, 5, 8, 12, 20, 28])
def test_cerny(ctx, n):
    d = cerny(n)
    r = ctx.solve(d, n, 2, EXACT)
    assert r.lower == r.upper == (n - 1) ** 2
    check_word(d, n, 2, r)


@pytest.mark.parametrize("n", [10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20])
def test_generate_hard_known_answers(ctx, n):
    # automaton.hpp:97-101
    expected = dict(zip(range(10, 21), [29, 35, 40, 44, 49, 54, 59, 63, 69, 76, 82]))[n]
    d = hard(n)
    r = ctx.solve(d, n, 2, EXACT)
    assert r.lower == r.upper == expected
    check_word(d, n, 2, r)


@pytest.mark.parametrize("n", [3, 4, 5, 6, 7])
def test_slowly_synchronizing_sink(ctx, n):
    d = slowlysink(n)
    r = ctx.solve(d, n, n - 1, EXACT)
    assert r.lower == r.upper == n * (n - 1) // 2
    check_word(d, n, n - 1, r)


@pytest.mark.parametrize("seed", range(1, 25))
def test_small_random_vs_brute(ctx, seed):
    n = 6 + seed % 12
    k = 2 + seed % 3
    d = random_dfa(n, k, 500 + seed)
    truth = oracle.brute(d, n, k)
    r = ctx.solve(d, n, k, EXACT)
    if truth < 0:
        assert r.non_synchro
    else:
        assert (r.lower, r.upper) == (truth, truth)
        check_word(d, n, k, r)


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_random_n200_exact(ctx, seed):
    n, k = 200, 2
    d = random_dfa(n, k, seed)
    r = ctx.solve(d, n, k, EXACT)
    ref = oracle.exact(d, n, k, oracle.ExactParams(threads=4))
    assert (r.lower, r.upper) == (ref.lower, ref.upper)
    check_word(d, n, k, r)


@pytest.mark.parametrize("n,seed", [(270, 1), (300, 4), (330, 12), (330, 13), (400, 34)])
def test_random_wide_rows_exact(ctx, n, seed):
    # five-, six- and seven-word rows (n = 257..448); seeds the oracle solves in seconds
    d = random_dfa(n, 2, seed)
    r = ctx.solve(d, n, 2, EXACT)
    ref = oracle.exact(d, n, 2, oracle.ExactParams(threads=8))
    assert (r.lower, r.upper) == (ref.lower, ref.upper)
    check_word(d, n, 2, r)


def cored_dfa(n, core, k, seed):
    """A random `core`-state automaton plus n - core transient states that map
    straight into the core: eight-word rows with a search the oracle finishes
    at once."""
    from synchrowords_gb300.generate import splitmix64
    g = splitmix64(seed)
    return list(random_dfa(core, k, seed)) + [next(g) % core for _ in range((n - core) * k)]


@pytest.mark.parametrize("n,core,k,seed", [(449, 60, 2, 7), (470, 60, 2, 8), (512, 80, 3, 9), (300, 100, 2, 10)])
def test_wide_rows_with_transient_states(ctx, n, core, k, seed):
    d = cored_dfa(n, core, k, seed)
    ref = oracle.exact(d, n, k, oracle.ExactParams(threads=8))
    for plan in (EXACT, BEAM_EXACT):
        r = ctx.solve(d, n, k, plan)
        assert (r.lower, r.upper) == (ref.lower, ref.upper)
        check_word(d, n, k, r)


@pytest.mark.parametrize("seed", [5, 6])
def test_random_n200_beam_exact(ctx, seed):
    n, k = 200, 2
    d = random_dfa(n, k, seed)
    r = ctx.solve(d, n, k, BEAM_EXACT)
    import math
    lg = math.log2(n)
    b = oracle.beam(d, n, k, oracle.BeamParams(dynamic=True, presort_indeg=True, min_beam_size=int(n * lg),
                                               max_beam_size=int(n * n * lg)), upper=(n - 1) ** 2 + 1)
    ex = oracle.exact(d, n, k, oracle.ExactParams(dfs_min_list_size=8192, bfs_small_list_size=n * k,
                                                  max_memory_mb=12 * 1024, threads=4), upper=b.upper)
    assert (r.lower, r.upper) == (ex.lower, ex.upper)
    check_word(d, n, k, r)


@pytest.mark.parametrize("seed", [1, 2, 3])
@pytest.mark.parametrize("dynamic", [False, True])
def test_beam_bound_matches_reference(ctx, seed, dynamic):
    import math
    n, k = 100, 3
    d = random_dfa(n, k, 70 + seed)
    lg = math.log2(n)
    cfg = {"presort": "indeg", "dynamic": dynamic, "beam_size": "AUT_N * std::log2(AUT_N)"}
    plan = json.dumps({"algorithms": [{"name": "Beam", "config": cfg}]})
    r = ctx.solve(d, n, k, plan)
    b = oracle.beam(d, n, k, oracle.BeamParams(beam_size=int(n * lg), dynamic=dynamic, presort_indeg=True))
    assert r.upper == b.upper
    if r.word is not None:
        check_word(d, n, k, r)


def test_non_synchronizing(ctx):
    # two disjoint cycles: no reset word
    n, k = 6, 2
    d = [1, 1, 2, 2, 0, 0, 4, 4, 5, 5, 3, 3]
    r = ctx.solve(d, n, k, EXACT)
    assert r.non_synchro


def test_single_state(ctx):
    r = ctx.solve([0, 0, 0, 0], 1, 4, EXACT)
    assert (r.lower, r.upper) == (0, 0)


@pytest.mark.parametrize("seed", [4])
def test_bounded_phase_in_chunks_under_a_small_budget(ctx, seed):
    # A 40 MB device budget ends the dominance-pruned search by memory a few
    # levels before the bound; the memory-bounded inverse phase then takes its
    # levels in chunks of 4096 parents (depth-first): the length must still be
    # exact and the word valid.
    n, k = 200, 2
    d = random_dfa(n, k, seed)
    plan = json.loads(BEAM_EXACT)
    plan["algorithms"][1]["config"].update({"max_memory_mb": 40, "dfs_min_list_size": 4096})
    r = ctx.solve(d, n, k, json.dumps(plan))
    ref = oracle.exact(d, n, k, oracle.ExactParams(threads=4))
    assert (r.lower, r.upper) == (ref.upper, ref.upper)
    check_word(d, n, k, r)
    assert r.stats["dfs_sets"] > 0


def test_solve_batch_concurrent_streams(ctx):
    autos = [(48, 2, random_dfa(48, 2, 900 + i)) for i in range(12)] + \
            [(100, 3, random_dfa(100, 3, 950 + i)) for i in range(4)] + [(28, 2, cerny(28))]
    res = ctx.solve_batch(autos, EXACT, workers=6)
    assert len(res) == len(autos)
    for (n, k, d), r in zip(autos, res):
        ref = oracle.exact(d, n, k)
        assert (r.lower, r.upper) == (ref.lower, ref.upper)
        check_word(d, n, k, r)


@pytest.mark.parametrize("n", [320, 384])
def test_c5_bench_automata_match_reference(ctx, n):
    """The eight n = 320 / 384 automata of the bench workloads, solved as the
    bench solves them (Beam(dynamic)+Exact, concurrent streams): lengths equal
    the compiled reference's (tests/golden/random_n{320,384}.json) and every
    word is verified."""
    g = json.loads((Path(__file__).resolve().parent / "golden" / f"random_n{n}.json").read_text())
    ref = g["reference"]["beam_exact"]
    autos = [(n, 2, random_dfa(n, 2, s)) for s in g["seeds"]]
    res = ctx.solve_batch(autos, json.dumps(ref["plan"]), workers=8)
    for (nn, k, d), r, want in zip(autos, res, ref["results"]):
        assert (r.lower, r.upper) == (want["lower"], want["upper"])
        check_word(d, nn, k, r)


def _fixture(name):
    return json.loads((Path(__file__).resolve().parent / "golden" / name).read_text())


@pytest.mark.parametrize("limit,cluster", [(104.0, 0), (-1.0, 0), (-1.0, -1)])
def test_c1_all_64_through_solve_batch_match_reference(native_lib, limit, cluster):
    """All 64 n = 48 automata of tests/golden/random_n48.json (the compiled
    reference's Exact lengths) through sw_solve_batch on each route: the
    shared-memory batched launch (the default for n = 48, as the bench's n48
    workload runs them), the cluster launch, and the worker streams."""
    import synchrowords_gb300 as sw
    g = _fixture("random_n48.json")
    want = g["reference"]["exact_default"]["results"]
    autos = [(48, 2, random_dfa(48, 2, s)) for s in g["seeds"]]
    assert len(autos) == 64
    with sw.Context(0) as c:
        c.set_batch_tuning(workers=8, batched_limit=limit, cluster_size=cluster)
        res = c.solve_batch(autos, EXACT)
        prof = c.last_batch_profile()
    if limit > 0:
        assert prof["small_solved"] == 64
    elif cluster >= 0:
        assert prof["cluster_solved"] == 64
    else:
        assert prof["streamed"] == 64
    for (n, k, d), r, w in zip(autos, res, want):
        assert (r.lower, r.upper) == (w["lower"], w["upper"])
        check_word(d, n, k, r)


@pytest.mark.parametrize("cluster", [0, 4, 16])
def test_c2_n200_cluster_launch_matches_reference(native_lib, cluster):
    """The sixteen n = 200 automata of the bench workload
    (tests/golden/random_n200.json, the compiled reference's plain Exact
    lengths) solved by the cluster launch alone: one cluster of 8 (default), 4
    or 16 CTAs per automaton, the whole search in one launch."""
    import synchrowords_gb300 as sw
    g = _fixture("random_n200.json")
    want = g["reference"]["exact_default"]["results"]
    autos = [(200, 2, random_dfa(200, 2, s)) for s in g["seeds"]]
    with sw.Context(0) as c:
        c.set_batch_tuning(workers=16, batched_limit=104.0, cluster_size=cluster, cluster_limit=1e9)
        res = c.solve_batch(autos, EXACT)
        prof = c.last_batch_profile()
    assert prof["cluster_solved"] == 16 and prof["streamed"] == 0, prof
    assert prof["launches"] == 1 and prof["device_ms"] > 0
    for (n, k, d), r, w in zip(autos, res, want):
        assert (r.lower, r.upper) == (w["lower"], w["upper"])
        check_word(d, n, k, r)


def test_cluster_launch_random_sizes_against_the_streamed_path(native_lib):
    """Uneven sizes across every set width of the cluster launch (n = 2..256,
    k = 1..16), against the streamed path (itself checked against the oracle
    and the reference's fixtures) and, for n <= 65, against the oracle;
    automata without a reset word fall through to the streamed path and are
    reported as such."""
    import random
    import synchrowords_gb300 as sw
    rng = random.Random(77)
    autos = []
    for i in range(48):
        n = rng.choice([2, 3, 17, 63, 64, 65, 100, 128, 129, 150, 192, 193, 230, 256])
        k = rng.choice([kk for kk in (1, 2, 3, 4, 7, 16) if n * kk <= (4096 if kk <= 2 else 520)])
        autos.append((n, k, random_dfa(n, k, 4000 + i)))
    with sw.Context(0) as c:
        c.set_batch_tuning(workers=8, batched_limit=-1.0, cluster_size=0, cluster_limit=1e9)
        res = c.solve_batch(autos, EXACT)
        prof = c.last_batch_profile()
        c.set_batch_tuning(workers=8, batched_limit=-1.0, cluster_size=-1)
        streamed = c.solve_batch(autos, EXACT)
    assert prof["cluster_solved"] > 24, prof
    for (n, k, d), r, s in zip(autos, res, streamed):
        assert (r.non_synchro, r.lower, r.upper) == (s.non_synchro, s.lower, s.upper), (n, k)
        if r.non_synchro:
            continue  # the reference's Exact has no such test: it reports its upper bound
        if n <= 65:
            ref = oracle.exact(d, n, k)
            assert (r.lower, r.upper) == (ref.lower, ref.upper), (n, k)
        if r.lower == r.upper:  # else both routes stopped at the plan's memory budget with the same bounds
            check_word(d, n, k, r)


LEARNED_EXACT = json.dumps({
    "upper_bound": "1ULL * (AUT_N - 1) * (AUT_N - 1) + 1",
    "algorithms": [
        {"name": "LearnedBeam", "config": {"beam_size": "4096", "order": "model"}},
        {"name": "Exact", "config": {"dfs_min_list_size": "8192", "bfs_small_list_size": "AUT_N * AUT_K",
                                     "dfs": True, "dfs_shortcut": True, "max_memory_mb": "12 * 1024"}}]})


@pytest.mark.parametrize("n", [320, 384])
def test_c5_learned_plan_matches_reference(ctx, n):
    """The sixteen n = 320 / 384 bench automata with the learned bound:
    LearnedBeam(4096, the packaged distance model) then the configs/exact.json
    Exact entry, as the bench's n384_learned workload runs them.  The bound only
    changes how the exact search proceeds: every length equals the compiled
    reference's (tests/golden/random_n{320,384}.json, Beam(dynamic)+Exact) and
    every word is verified."""
    import synchrowords_gb300 as sw
    if not sw.DEFAULT_MODEL.exists():
        pytest.skip("no packaged model")
    g = _fixture(f"random_n{n}.json")
    ref = g["reference"]["beam_exact"]
    autos = [(n, 2, random_dfa(n, 2, s)) for s in g["seeds"]]
    res = ctx.solve_batch(autos, LEARNED_EXACT, workers=8)
    for (nn, k, d), r, want in zip(autos, res, ref["results"]):
        assert (r.lower, r.upper) == (want["lower"], want["upper"])
        assert r.runs[0][0] == "LearnedBeam"
        check_word(d, nn, k, r)
