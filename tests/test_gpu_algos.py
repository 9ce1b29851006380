"""Eppstein and Brute on the GPU against the reference's golden outputs
(tests/golden/eppstein.json, brute.json) and the oracle."""
import json
from pathlib import Path

import pytest

import oracle
from synchrowords_gb300.generate import cerny, random_dfa

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"


def plan(name, cfg=None, **top):
    return json.dumps(dict({"algorithms": [{"name": name, "config": cfg or {}}]}, **top))


def verified(d, n, k, r):
    assert r.word is not None and len(r.word) == r.upper
    assert len(oracle.apply_word(d, n, k, r.word)) == 1


def eppstein_cases():
    return json.loads((GOLD / "eppstein.json").read_text())["cases"]


@pytest.mark.parametrize("case", eppstein_cases(), ids=lambda c: f"n{c['n']}k{c['k']}s{c['seed']}")
def test_eppstein_matches_reference(ctx, case):
    n, k = case["n"], case["k"]
    d = case["delta"] or random_dfa(n, k, case["seed"])
    top = {"upper_bound": case["upper_bound"]} if "upper_bound" in case else {}
    r = ctx.solve(d, n, k, plan("Eppstein", {"find_word": True}, **top))
    ref = case["reference"]
    if ref.get("non_synchro"):
        assert r.non_synchro
        return
    assert (r.lower, r.upper) == (ref["lower"], ref["upper"])
    if "word" in ref:
        assert r.word == ref["word"]  # same pair choices, same letters
        verified(d, n, k, r)


@pytest.mark.parametrize("seed", range(1, 9))
def test_eppstein_random_vs_oracle(ctx, seed):
    n, k = [(33, 2), (70, 3), (130, 2), (257, 2), (500, 2), (64, 4), (16, 16), (511, 3)][seed - 1]
    d = random_dfa(n, k, 4000 + seed)
    r = ctx.solve(d, n, k, plan("Eppstein"))
    o, w = oracle.eppstein(d, n, k)
    assert (r.lower, r.upper, r.non_synchro) == (o.lower, o.upper, o.non_synchro)
    if not o.non_synchro:
        assert r.word == w
        verified(d, n, k, r)


def test_eppstein_then_exact(ctx):
    # the Eppstein bound and word feed the exact search, whose length must not change
    n, k = 120, 2
    d = random_dfa(n, k, 77)
    two = json.dumps({"algorithms": [{"name": "Eppstein", "config": {}}, {"name": "Exact", "config": {}}]})
    r = ctx.solve(d, n, k, two)
    ref = oracle.exact(d, n, k, oracle.ExactParams(threads=4))
    assert (r.lower, r.upper) == (ref.lower, ref.upper)
    verified(d, n, k, r)


def brute_cases():
    return json.loads((GOLD / "brute.json").read_text())["cases"]


@pytest.mark.parametrize("case", brute_cases(), ids=lambda c: f"n{c['n']}k{c['k']}s{c['seed']}")
def test_brute_matches_reference(ctx, case):
    n, k = case["n"], case["k"]
    d = random_dfa(n, k, case["seed"])
    r = ctx.solve(d, n, k, plan("Brute", {"max_n": "24"}))
    ref = case["reference"]
    if ref.get("non_synchro"):
        assert r.non_synchro
        return
    assert (r.lower, r.upper) == (ref["lower"], ref["upper"])
    verified(d, n, k, r)


@pytest.mark.parametrize("n", [2, 5, 13, 20, 28])
def test_brute_cerny(ctx, n):
    d = cerny(n)
    r = ctx.solve(d, n, 2, plan("Brute", {"max_n": "32"}, upper_bound="100000"))
    assert r.lower == r.upper == (n - 1) ** 2
    verified(d, n, 2, r)


@pytest.mark.parametrize("seed", range(1, 7))
def test_brute_random_vs_exact(ctx, seed):
    n, k = [(26, 2), (28, 2), (30, 2), (32, 2), (27, 3), (32, 3)][seed - 1]
    d = random_dfa(n, k, 6100 + seed)
    r = ctx.solve(d, n, k, plan("Brute", {"max_n": "32"}))
    e = ctx.solve(d, n, k, plan("Exact"))
    assert (r.lower, r.upper, r.non_synchro) == (e.lower, e.upper, e.non_synchro)
    if not r.non_synchro:
        verified(d, n, k, r)


def test_brute_limits(ctx):
    d = random_dfa(30, 2, 1)
    # n above max_n: skipped, bounds untouched
    r = ctx.solve(d, 30, 2, plan("Brute"))
    assert (r.lower, r.upper) == (0, 30 ** 3 // 6)
    # max_n above 32: refused, bounds untouched
    r = ctx.solve(d, 30, 2, plan("Brute", {"max_n": "40"}))
    assert (r.lower, r.upper) == (0, 30 ** 3 // 6)
    # non-synchronizing
    r = ctx.solve([1, 1, 2, 2, 0, 0, 4, 4, 5, 5, 3, 3], 6, 2, plan("Brute"))
    assert r.non_synchro
