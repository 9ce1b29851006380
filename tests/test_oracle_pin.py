"""Pin the oracle (the CPU restatement of the reference in oracle/) to the
reference: committed golden vectors generated by the compiled reference
(tests/golden/make_golden.py), the reference's known-answer material
(README example, Černý, generate_hard, slowly-synchronizing family), an
independent power-set BFS, and — where the reference checkout exists — the
reference binary itself."""
import json
import math
import os
from pathlib import Path

import pytest

import oracle
from synchrowords_gb300 import generate as gen

GOLD = Path(__file__).resolve().parent / "golden"


def load(name):
    return json.loads((GOLD / name).read_text())


def checksum(autos):
    import hashlib
    h = hashlib.sha256()
    for n, k, d in autos:
        h.update(f"{k} {n}:".encode() + ",".join(map(str, d)).encode() + b";")
    return h.hexdigest()[:16]


def test_generator_pinned_by_fixture_checksums():
    for name in ("random_n48.json", "random_n200.json"):
        g = load(name)
        autos = [(g["n"], g["k"], gen.random_dfa(g["n"], g["k"], s)) for s in g["seeds"]]
        assert checksum(autos) == g["checksum"], name


def test_splitmix64_known_values():
    # SplitMix64 of seed 0 (the published reference sequence)
    g = gen.splitmix64(0)
    assert [next(g) for _ in range(3)] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_oracle_matches_reference_n48_lengths_and_traces():
    g = load("random_n48.json")
    ref = g["reference"]["exact_default"]
    for seed, r, tr in zip(g["seeds"], ref["results"], ref["traces"]):
        d = gen.random_dfa(48, 2, seed)
        o = oracle.exact(d, 48, 2, trace_capacity=4096)
        assert (o.lower, o.upper) == (r["lower"], r["upper"]), seed
        mine = [list(s) for s in o.trace if s[0] in (0, 1)]
        assert mine == tr, f"per-step frontier sizes differ for seed {seed}"


def test_oracle_matches_reference_n200_subset():
    g = load("random_n200.json")
    ref = g["reference"]["exact_default"]
    for seed, r, tr in list(zip(g["seeds"], ref["results"], ref["traces"]))[:3]:
        d = gen.random_dfa(200, 2, seed)
        o = oracle.exact(d, 200, 2, oracle.ExactParams(threads=4), trace_capacity=4096)
        assert (o.lower, o.upper) == (r["lower"], r["upper"]), seed
        assert [list(s) for s in o.trace if s[0] in (0, 1)] == tr, seed


def test_oracle_matches_reference_beam_exact_n200_subset():
    g = load("random_n200.json")
    ref = g["reference"]["beam_exact"]
    n, k = 200, 2
    lg = math.log2(n)
    for seed, r in list(zip(g["seeds"], ref["results"]))[:3]:
        d = gen.random_dfa(n, k, seed)
        b = oracle.beam(d, n, k, oracle.BeamParams(dynamic=True, presort_indeg=True, min_beam_size=int(n * lg),
                                                   max_beam_size=int(n * n * lg)), upper=(n - 1) ** 2 + 1)
        e = oracle.exact(d, n, k, oracle.ExactParams(dfs_min_list_size=8192, bfs_small_list_size=n * k,
                                                     max_memory_mb=12 * 1024, threads=4), upper=b.upper)
        assert (e.lower, e.upper) == (r["lower"], r["upper"]), seed


def test_oracle_beam_matches_reference():
    for c in load("beam.json")["cases"]:
        n, k = c["n"], c["k"]
        d = gen.random_dfa(n, k, c["seed"])
        o = oracle.beam(d, n, k, oracle.BeamParams(beam_size=int(n * math.log2(n)), presort_indeg=True))
        assert o.upper == c["reference"]["upper"], c


def test_known_answer_families():
    fam = load("families.json")
    for e in fam["cerny"]:
        if e["n"] <= 24:
            assert oracle.exact(gen.cerny(e["n"]), e["n"], 2).upper == e["expected"]
    for e in fam["cerny_ref"]:
        if e["n"] <= 24:
            assert oracle.exact(gen.cerny_ref(e["n"]), e["n"], 2).upper == e["expected"]
    for e in fam["hard"]:
        assert oracle.exact(gen.hard(e["n"]), e["n"], 2).upper == e["expected"]
    for e in fam["slowlysink"]:
        assert oracle.exact(gen.slowlysink(e["n"]), e["n"], e["n"] - 1).upper == e["expected"]


def test_readme_example():
    g = load("readme.json")
    for a, exp in zip(g["automata"], g["expected"]):
        n, k, d = a["n"], a["k"], a["delta"]
        if exp.get("non_synchro"):
            assert oracle.brute(d, n, k) == -1
            continue
        o = oracle.exact(d, n, k)
        assert (o.lower, o.upper) == (exp["lower"], exp["upper"])


@pytest.mark.parametrize("seed", range(40))
def test_oracle_vs_power_set_bfs(seed):
    n = 3 + seed % 14
    k = 2 + seed % 3
    d = gen.random_dfa(n, k, 7000 + seed)
    truth = oracle.brute(d, n, k)
    if truth < 0:
        pytest.skip("not synchronizing")
    o = oracle.exact(d, n, k)
    assert (o.lower, o.upper) == (truth, truth)


# the reference checkout the recipe compiles from (SYNCHRO_REF_ROOT, or the
# recipe's own default location); absent on machines without it
from oracle.build_ref import REF_ROOT as REF  # noqa: E402


@pytest.mark.skipif(not REF.is_dir(), reason="reference checkout not present")
@pytest.mark.slow
def test_oracle_matches_compiled_reference_random_n24():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLD / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    autos = [(24, 3, gen.random_dfa(24, 3, 300 + i)) for i in range(12)]
    res, _ = mg.run_reference({"algorithms": [{"name": "Exact", "config": {}}]}, autos)
    for (n, k, d), r in zip(autos, res):
        o = oracle.exact(d, n, k)
        assert (o.lower, o.upper) == (r["lower"], r["upper"])


def test_oracle_matches_reference_edge_fixture():
    """One-letter, two-state, permutation, Cerny and width-boundary automata:
    the oracle's Exact bounds equal the compiled reference's (for automata
    without a reset word both report the upper bound)."""
    for c in load("batch_edges.json")["cases"]:
        o = oracle.exact(c["delta"], c["n"], c["k"])
        assert (o.lower, o.upper) == (c["reference"]["lower"], c["reference"]["upper"]), (c["n"], c["k"])


def test_oracle_eppstein_matches_reference_fixture():
    g = load("eppstein.json")
    for c in g["cases"]:
        n, k = c["n"], c["k"]
        d = c["delta"] or gen.random_dfa(n, k, c["seed"])
        upper = int(c["upper_bound"]) if "upper_bound" in c else None
        o, w = oracle.eppstein(d, n, k, upper=upper)
        r = c["reference"]
        if r.get("non_synchro"):
            assert o.non_synchro
            continue
        assert (o.lower, o.upper) == (r["lower"], r["upper"])
        assert w == r.get("word")


def test_oracle_brute_matches_reference_fixture():
    for c in load("brute.json")["cases"]:
        d = gen.random_dfa(c["n"], c["k"], c["seed"])
        want = oracle.brute(d, c["n"], c["k"])
        r = c["reference"]
        assert (want < 0) == bool(r.get("non_synchro"))
        if want >= 0:
            assert (r["lower"], r["upper"]) == (want, want)


def test_mlp_oracle_backward_matches_finite_differences():
    """The numpy restatement of the distance model (the checker of the GPU
    gradients) is itself checked: without bf16 rounding, in float64, its
    backward pass matches central differences of its forward pass."""
    import numpy as np
    from oracle import mlp
    rng = np.random.default_rng(11)
    n = 23
    feat = rng.normal(size=(n, mlp.FEAT))
    bits = (rng.random((40, n)) < 0.4).astype(np.float64)
    t = rng.normal(10.0, 3.0, size=40)
    p = rng.normal(0, 0.2, size=mlp.PARAMS)
    mlp.EXACT = True
    try:
        _, cache = mlp.forward(p, feat, bits)
        g, _ = mlp.backward(cache, t)

        def loss(q):
            y, _ = mlp.forward(q, feat, bits)
            return float(np.mean((y - t) ** 2))

        idx = list(rng.choice(mlp.PARAMS, 60, replace=False)) + [mlp.OFF["b3"][0], mlp.OFF["c"][0] + 3]
        for i in idx:
            e = np.zeros(mlp.PARAMS)
            e[i] = 1e-5
            num = (loss(p + e) - loss(p - e)) / 2e-5
            assert abs(num - g[i]) <= 1e-5 + 1e-4 * abs(num), (i, num, g[i])
    finally:
        mlp.EXACT = False


def test_bf16_rounding_is_nearest_even():
    import numpy as np
    from oracle import mlp
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -7 + 2 ** -9, -2.5e-3], dtype=np.float32)
    # ties go to the even mantissa; 7 fraction bits near 1
    assert mlp.bf16(x).tolist() == [1.0, 1.0, 1.0 + 2 ** -6, 1.0 + 2 ** -7, -0.00250244140625]
