"""Uneven batch of 4096 random automata, n ~ U[32,160], k ~ U{2,3}, solved
through sw_solve_batch (the shared-memory batched launch, the cluster launch
and worker streams); every length equals the
committed golden (oracle, spot-checked against the compiled reference) and every
word is verified."""
import json
from pathlib import Path

import pytest

import oracle
from synchrowords_gb300 import generate as gen

pytestmark = pytest.mark.gpu

GOLD = json.loads((Path(__file__).resolve().parent / "golden" / "batch_4096.json").read_text())
PLAN = json.dumps({"algorithms": [{"name": "Exact", "config": {}}]})


def test_batch_4096_lengths_and_words(ctx):
    autos = gen.batch(GOLD["count"], GOLD["seed"])
    res = ctx.solve_batch(autos, PLAN, workers=16)
    prof = ctx.last_batch_profile()
    # with the default tuning both device launches take part and the streams see only leftovers
    assert prof["small_solved"] > 1000 and prof["cluster_solved"] > 1000, prof
    non_sync = set(GOLD["non_synchronizing_indices"])
    for i, ((n, k, d), r, L) in enumerate(zip(autos, res, GOLD["lengths"])):
        if i in non_sync:
            assert r.non_synchro, i
            continue
        assert (r.lower, r.upper) == (L, L), (i, n, k, r.lower, r.upper, L)
        assert r.word is not None and len(r.word) == L
        assert len(oracle.apply_word(d, n, k, r.word)) == 1, i


def check_against_golden(autos, res):
    non_sync = set(GOLD["non_synchronizing_indices"])
    for i, ((n, k, d), r) in enumerate(zip(autos, res)):
        L = GOLD["lengths"][i]
        if i in non_sync:
            assert r.non_synchro, i
            continue
        assert (r.lower, r.upper) == (L, L), (i, n, k, r.lower, r.upper, L)
        assert r.word is not None and len(oracle.apply_word(d, n, k, r.word)) == 1, i


def test_autotune_batch_picks_candidates_and_keeps_results(native_lib):
    import synchrowords_gb300 as sw
    ctx = sw.Context(0)  # its own context: the tuning stays with it
    assert ctx.get_batch_tuning() == {"workers": 0, "batched_limit": 104.0, "cluster_size": 0,
                                      "cluster_limit": sw.DEFAULT_CLUSTER_LIMIT}
    autos = gen.batch(GOLD["count"], GOLD["seed"])[:200]
    tuned = ctx.autotune_batch(autos, PLAN, workers=(2, 6), limits=(-1.0, 104.0), reps=1)
    assert tuned["workers"] in (2, 6) and tuned["batched_limit"] in (-1.0, 104.0)
    assert set(tuned["ms"]["workers"]) == {2, 6} and set(tuned["ms"]["batched_limit"]) == {-1.0, 104.0}
    assert all(t > 0 for d in tuned["ms"].values() for t in d.values())
    assert ctx.get_batch_tuning() == {"workers": tuned["workers"], "batched_limit": tuned["batched_limit"],
                                      "cluster_size": 0,
                                      "cluster_limit": sw.DEFAULT_CLUSTER_LIMIT}
    check_against_golden(autos, ctx.solve_batch(autos, PLAN))  # workers = 0: the tuned count
    # every route gives the same answers: worker streams only, the shared-memory
    # launch for all it accepts, the cluster launch for all, and clusters of 4 and 16 CTAs
    for limit, cs in ((-1.0, -1), (1024.0, -1), (-1.0, 0), (-1.0, 4), (-1.0, 16)):
        ctx.set_batch_tuning(workers=4, batched_limit=limit, cluster_size=cs, cluster_limit=1e9)
        check_against_golden(autos, ctx.solve_batch(autos, PLAN))
        prof = ctx.last_batch_profile()
        if cs >= 0:
            assert prof["cluster_solved"] > 0 and prof["small_solved"] == 0, prof
    # the cluster autotuner: candidates timed, the choice kept, answers unchanged
    tuned = ctx.autotune_cluster(autos, PLAN, sizes=(4, 8), limits=(-1.0, 160.0), reps=1)
    assert tuned["cluster_size"] in (4, 8) and tuned["cluster_limit"] in (-1.0, 160.0)
    assert set(tuned["ms"]["cluster_size"]) == {4, 8} and set(tuned["ms"]["cluster_limit"]) == {-1.0, 160.0}
    assert ctx.get_batch_tuning()["cluster_size"] == tuned["cluster_size"]
    check_against_golden(autos, ctx.solve_batch(autos, PLAN))
    ctx.close()


def test_repeated_batch_replays_its_captured_round(native_lib):
    """A batch of a shape seen before replays the device round captured into a
    CUDA graph for it; a batch of another shape captures its own; answers stay
    those of the golden file."""
    import synchrowords_gb300 as sw
    ctx = sw.Context(0)
    try:
        autos = gen.batch(GOLD["count"], GOLD["seed"])[:300]
        first = ctx.solve_batch(autos, PLAN, workers=4)
        p1 = ctx.last_batch_profile()
        assert p1["graph_replays"] == 0 and p1["small_solved"] > 0 and p1["cluster_solved"] > 0, p1
        check_against_golden(autos, first)
        again = ctx.solve_batch(autos, PLAN, workers=4)
        p2 = ctx.last_batch_profile()
        assert p2["graph_replays"] >= 1 and p2["launches"] == p1["launches"], (p1, p2)
        # which shortest word a persistent launch finds first may vary between runs; lengths may not
        assert [(r.lower, r.upper) for r in again] == [(r.lower, r.upper) for r in first]
        check_against_golden(autos, again)
        other = autos[:120]
        check_against_golden(other, ctx.solve_batch(other, PLAN, workers=4))
        assert ctx.last_batch_profile()["graph_replays"] == 0
        check_against_golden(autos, ctx.solve_batch(autos, PLAN, workers=4))
        assert ctx.last_batch_profile()["graph_replays"] >= 1
    finally:
        ctx.close()
