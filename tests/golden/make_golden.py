"""Generate the golden fixtures under tests/golden/ from the compiled reference.

Run here, where the reference checkout exists (it does not travel to the GPU
machine); the JSON files it writes are committed and read by the tests.

    python tests/golden/make_golden.py [--big]

Every automaton is regenerated from its seed by synchrowords_gb300.generate
(SplitMix64), so a fixture stores seeds and answers, plus a checksum of the
generated transition tables that pins the generator.  Answers come from the
reference binary built by oracle/build_ref.py from the reference's own
sources; the oracle (the CPU restatement) is run on the same inputs and must
agree before anything is written.  `--big` adds the n = 320 / 384 fixtures
(several minutes of reference CPU time).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import math
import re
import subprocess
import sys
import tempfile
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from oracle import build_ref  # noqa: E402
from synchrowords_gb300 import generate as gen  # noqa: E402

REF = build_ref.REF_ROOT

EXACT_DEFAULT = {"algorithms": [{"name": "Exact", "config": {}}]}
# configs/exact.json without the Brute / Eppstein entries
BEAM_EXACT = {
    "upper_bound": "1ULL * (AUT_N - 1) * (AUT_N - 1) + 1",
    "algorithms": [
        {"name": "Beam", "config": {"presort": "indeg", "dynamic": True,
                                    "min_beam_size": "AUT_N * std::log2(AUT_N)",
                                    "max_beam_size": "AUT_N * AUT_N * std::log2(AUT_N)",
                                    "beam_exact_ratio": 0.01}},
        {"name": "Exact", "config": {"dfs_min_list_size": "8192", "bfs_small_list_size": "AUT_N * AUT_K",
                                     "dfs": True, "dfs_shortcut": True, "max_memory_mb": "12 * 1024"}}]}
BEAM_ONLY = {"algorithms": [{"name": "Beam", "config": {"presort": "indeg",
                                                         "beam_size": "AUT_N * std::log2(AUT_N)"}}]}


def checksum(autos) -> str:
    h = hashlib.sha256()
    for n, k, d in autos:
        h.update(f"{k} {n}:".encode() + ",".join(map(str, d)).encode() + b";")
    return h.hexdigest()[:16]


def run_reference(plan: dict, autos, threads: int = 1, level: int = 3):
    """Run the reference on automata of one (n, k); returns [(lb, ub, ms dict, trace)]."""
    n, k = autos[0][0], autos[0][1]
    assert all(a[0] == n and a[1] == k for a in autos)
    binary = build_ref.build(n, k, plan, threads)
    with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
        f.write(gen.to_text(autos))
        path = f.name
    r = subprocess.run([str(binary), "-f", path, "-L", str(level)], capture_output=True, text=True, check=True)
    results = []
    traces, cur = [], []
    for line in r.stderr.splitlines():
        m = re.search(r"\((I?BFS)\)(?: \[novisited\])? len: (\d+) list size: (\d+) inv list size: (\d+)", line)
        if m:
            cur.append([0 if m.group(1) == "BFS" else 1, int(m.group(2)), int(m.group(3)), int(m.group(4))])
        if "mlsw" in line:
            traces.append(cur)
            cur = []
    for i, line in enumerate(r.stdout.splitlines()):
        m = re.match(r"(\d+): \[(\d+), (\d+)\] \((.*)\)", line)
        if m:
            ms = {a: int(t) for a, t in re.findall(r"\((\w+), (\d+)\)", m.group(4))}
            res = {"lower": int(m.group(2)), "upper": int(m.group(3)), "ms": ms}
            w = re.search(r"\{([\d ]*)\}\s*$", line)
            if w:
                res["word"] = [int(x) for x in w.group(1).split()]
            results.append(res)
        elif "NON SYNCHRO" in line:
            results.append({"non_synchro": True})
    return results, traces


def oracle_beam_exact(d, n, k, threads=1):
    lg = math.log2(n)
    ub = (n - 1) ** 2 + 1
    b = oracle.beam(d, n, k, oracle.BeamParams(dynamic=True, presort_indeg=True, min_beam_size=int(n * lg),
                                               max_beam_size=int(n * n * lg)), upper=ub)
    e = oracle.exact(d, n, k, oracle.ExactParams(dfs_min_list_size=8192, bfs_small_list_size=n * k,
                                                 max_memory_mb=12 * 1024, threads=threads), upper=b.upper)
    return b.upper, e


def write(name: str, obj, compact: bool = False) -> None:
    (HERE / name).write_text(json.dumps(obj, indent=None if compact else 1, sort_keys=True) + "\n")
    print("wrote", name)


def fixture_random(name, n, k, seeds, plans, threads=1, with_trace=False):
    autos = [(n, k, gen.random_dfa(n, k, s)) for s in seeds]
    out = {"generator": "random_dfa(n, k, seed)", "n": n, "k": k, "seeds": list(seeds),
           "checksum": checksum(autos), "reference": {}}
    for pname, plan in plans.items():
        t0 = time.time()
        res, traces = run_reference(plan, autos, threads)
        out["reference"][pname] = {"plan": plan, "threads": threads, "results": res,
                                   "seconds": round(time.time() - t0, 1)}
        if with_trace:
            out["reference"][pname]["traces"] = traces
        # the oracle must agree before the fixture is written
        for (nn, kk, d), r in zip(autos, res):
            if pname == "exact_default":
                o = oracle.exact(d, nn, kk, oracle.ExactParams(threads=threads))
                assert (o.lower, o.upper) == (r["lower"], r["upper"]), (pname, r, o)
            elif pname == "beam_exact":
                _, o = oracle_beam_exact(d, nn, kk, threads)
                assert (o.lower, o.upper) == (r["lower"], r["upper"]), (pname, r, o)
    write(name, out)


def fixture_families():
    fam = {"cerny": [], "cerny_ref": [], "hard": [], "slowlysink": []}
    for n in range(2, 31):
        fam["cerny"].append({"n": n, "expected": (n - 1) ** 2})
        fam["cerny_ref"].append({"n": n, "expected": (n - 1) ** 2})
    # automaton.hpp:97-101
    for n, v in zip(range(10, 21), [29, 35, 40, 44, 49, 54, 59, 63, 69, 76, 82]):
        fam["hard"].append({"n": n, "expected": v})
    for n in range(3, 11):
        fam["slowlysink"].append({"n": n, "expected": n * (n - 1) // 2})
    # cross-check a few with the reference binary itself
    checks = [("cerny", 28, 2, gen.cerny(28)), ("cerny_ref", 28, 2, gen.cerny_ref(28)),
              ("hard", 20, 2, gen.hard(20)), ("slowlysink", 8, 7, gen.slowlysink(8))]
    verified = []
    for fname, n, k, d in checks:
        res, _ = run_reference(EXACT_DEFAULT, [(n, k, d)])
        verified.append({"family": fname, "n": n, "reference": res[0]})
        exp = {"cerny": (n - 1) ** 2, "cerny_ref": (n - 1) ** 2, "hard": 82, "slowlysink": n * (n - 1) // 2}[fname]
        assert res[0]["upper"] == exp == res[0]["lower"], (fname, res)
    fam["reference_verified"] = verified
    write("families.json", fam)


def fixture_readme():
    text = (REF / "data" / "readme_input.txt").read_text()
    toks = text.split()
    autos = []
    i = 0
    while i < len(toks):
        k, n = int(toks[i]), int(toks[i + 1])
        d = [int(x) for x in toks[i + 2:i + 2 + n * k]]
        autos.append({"n": n, "k": k, "delta": d})
        i += 2 + n * k
    # docs/install.md:103-106 (expected output file of the README run)
    expected = [{"lower": 0, "upper": 0}, {"non_synchro": True}, {"lower": 3, "upper": 3},
                {"lower": 18, "upper": 18}]
    # confirm #3 with the reference's Exact (without the Reduce pre-pass)
    a = autos[3]
    res, _ = run_reference(EXACT_DEFAULT, [(a["n"], a["k"], a["delta"])])
    assert (res[0]["lower"], res[0]["upper"]) == (18, 18), res
    write("readme.json", {"source": "data/readme_input.txt; expected lines docs/install.md:103-106",
                          "automata": autos, "expected": expected})


def fixture_beam():
    out = {"cases": []}
    for n, k, seed in [(100, 3, 71), (100, 3, 72), (100, 3, 73), (150, 2, 11), (200, 2, 21)]:
        d = gen.random_dfa(n, k, seed)
        res, _ = run_reference(BEAM_ONLY, [(n, k, d)])
        o = oracle.beam(d, n, k, oracle.BeamParams(beam_size=int(n * math.log2(n)), presort_indeg=True))
        assert o.upper == res[0]["upper"], (res, o)
        out["cases"].append({"n": n, "k": k, "seed": seed, "plan": BEAM_ONLY, "reference": res[0]})
    write("beam.json", out)


def fixture_batch(count=4096, seed=2026, sample=24):
    autos = gen.batch(count, seed)
    lengths = []
    t0 = time.time()
    for n, k, d in autos:
        r = oracle.exact(d, n, k, oracle.ExactParams(threads=4))
        lengths.append([r.lower, r.upper])
    oracle_s = time.time() - t0
    # spot-check against the reference binary on a sample spread over (n, k)
    idx = sorted(range(count), key=lambda i: (autos[i][0], autos[i][1]))[:: max(1, count // sample)][:sample]
    checked = []
    for i in idx:
        n, k, d = autos[i]
        res, _ = run_reference(EXACT_DEFAULT, [(n, k, d)])
        assert [res[0]["lower"], res[0]["upper"]] == lengths[i], (i, res, lengths[i])
        checked.append(i)
    write("batch_4096.json", {"generator": "batch(4096, 2026): n ~ U[32,160], k ~ U{2,3}", "count": count,
                              "seed": seed, "checksum": checksum(autos), "lengths": lengths,
                              "answers_from": "oracle (trace-identical restatement of the reference)",
                              "reference_checked_indices": checked, "oracle_seconds": round(oracle_s, 1)},
          compact=True)


def fixture_batch_more_checks(extra=104):
    """Check `extra` more automata of the 4096 batch against the reference
    binary (spread over (n, k), none checked before) and record them."""
    path = HERE / "batch_4096.json"
    g = json.loads(path.read_text())
    autos = gen.batch(g["count"], g["seed"])
    assert checksum(autos) == g["checksum"]
    done = set(g["reference_checked_indices"])
    order = [i for i in sorted(range(len(autos)), key=lambda i: (autos[i][0], autos[i][1], i)) if i not in done]
    pick = order[:: max(1, len(order) // extra)][:extra]
    for i in pick:
        n, k, d = autos[i]
        res, _ = run_reference(EXACT_DEFAULT, [(n, k, d)])
        assert res[0]["lower"] == res[0]["upper"] == g["lengths"][i], (i, res, g["lengths"][i])
        done.add(i)
    g["reference_checked_indices"] = sorted(done)
    write("batch_4096.json", g, compact=True)


def edge_automata():
    """One-letter and two-state automata, permutation automata (no reset
    word), Cerny automata up to 24 states, and random automata at every set
    width boundary from 33 to 256 states."""
    import random
    rng = random.Random(77)
    autos = []
    for n in (2, 3, 5, 9):
        for _ in range(3):
            autos.append((n, 1, [rng.randrange(n) for _ in range(n)]))
    for k in (1, 2, 3, 4):
        for _ in range(2):
            autos.append((2, k, [rng.randrange(2) for _ in range(2 * k)]))
    for n, k in ((6, 2), (20, 3), (70, 2)):
        d = [0] * (n * k)
        for a in range(k):
            p = list(range(n))
            rng.shuffle(p)
            for q in range(n):
                d[q * k + a] = p[q]
        autos.append((n, k, d))
    for n in (5, 12, 20, 24):
        autos.append((n, 2, gen.cerny(n)))
    for n, k, s in ((33, 2, 1), (64, 3, 2), (65, 2, 3), (100, 2, 4), (128, 2, 5), (129, 2, 6), (150, 2, 7),
                    (192, 2, 8), (193, 2, 9), (230, 2, 10), (256, 2, 12), (90, 4, 13)):
        autos.append((n, k, gen.random_dfa(n, k, 5000 + s)))
    return autos


def fixture_edges():
    autos = edge_automata()
    cases = []
    for n, k, d in autos:
        res, _ = run_reference(EXACT_DEFAULT, [(n, k, d)])
        r = res[0]
        o = oracle.exact(d, n, k)
        if not r.get("non_synchro"):
            assert (o.lower, o.upper) == (r["lower"], r["upper"]), (n, k, r, o)
        cases.append({"n": n, "k": k, "delta": d, "reference": {x: r[x] for x in ("lower", "upper", "non_synchro")
                                                                 if x in r}})
    write("batch_edges.json", {"plan": EXACT_DEFAULT, "source": "edge_automata() in make_golden.py",
                               "cases": cases})


EPPSTEIN = {"algorithms": [{"name": "Eppstein", "config": {"find_word": True}}]}


def fixture_eppstein():
    """Eppstein bounds and words from the reference (find_word on)."""
    cases = []
    inputs = [(n, k, seed, gen.random_dfa(n, k, seed)) for n, k, seed in
              [(5, 2, 1), (12, 2, 2), (12, 3, 3), (30, 2, 4), (48, 2, 5), (64, 2, 6), (100, 2, 7), (100, 3, 8),
               (200, 2, 9), (320, 2, 10), (384, 2, 11)]]
    inputs += [(n, 2, None, gen.cerny(n)) for n in (4, 10, 20)]
    inputs += [(6, 2, None, [1, 1, 2, 2, 0, 0, 4, 4, 5, 5, 3, 3])]  # two cycles: not synchronizing
    for n, k, seed, d in inputs:
        res, _ = run_reference(EPPSTEIN, [(n, k, d)])
        r = res[0]
        o, w = oracle.eppstein(d, n, k)
        if r.get("non_synchro"):
            assert o.non_synchro, (n, seed)
        else:
            assert (o.lower, o.upper) == (r["lower"], r["upper"]), (n, seed, r, o)
            assert w == r.get("word"), (n, seed)
        cases.append({"n": n, "k": k, "seed": seed, "delta": d if seed is None else None, "reference": r})
    # a bound below the greedy length leaves the bounds unchanged (eppstein.hpp:104-106)
    tight = dict(EPPSTEIN, upper_bound="5")
    d = gen.random_dfa(48, 2, 5)
    res, _ = run_reference(tight, [(48, 2, d)])
    o, _ = oracle.eppstein(d, 48, 2, upper=5)
    assert (o.lower, o.upper) == (res[0]["lower"], res[0]["upper"]) == (0, 5)
    cases.append({"n": 48, "k": 2, "seed": 5, "delta": None, "upper_bound": "5", "reference": res[0]})
    write("eppstein.json", {"plan": EPPSTEIN, "cases": cases})


BRUTE = {"algorithms": [{"name": "Brute", "config": {"max_n": "24"}}]}


def fixture_brute():
    """Brute lengths from the reference for n <= 24."""
    cases = []
    for n, k, seed in [(6, 2, 1), (9, 3, 2), (12, 2, 3), (16, 2, 4), (18, 3, 5), (20, 2, 6), (22, 2, 7),
                       (24, 2, 8), (24, 3, 9)]:
        d = gen.random_dfa(n, k, seed)
        res, _ = run_reference(BRUTE, [(n, k, d)])
        want = oracle.brute(d, n, k)
        r = res[0]
        assert (want < 0 and r.get("non_synchro")) or (r["lower"], r["upper"]) == (want, want), (n, seed, r, want)
        cases.append({"n": n, "k": k, "seed": seed, "reference": r})
    write("brute.json", {"plan": BRUTE, "cases": cases})


REDUCE_ONLY = {"algorithms": [{"name": "Reduce", "config": {}}]}


def reference_reduce(plan, n, k, d):
    """Reduce on the reference: (bounds line, reduced N, BFS steps) from its log."""
    binary = build_ref.build(n, k, plan)
    with tempfile.NamedTemporaryFile("w", suffix=".txt", delete=False) as f:
        f.write(gen.to_text([(n, k, d)]))
        path = f.name
    r = subprocess.run([str(binary), "-f", path, "-L", "2"], capture_output=True, text=True, check=True)
    m = re.search(r"Reduced to N = (\d+) in (\d+) bfs steps", r.stderr)
    line = re.match(r"\d+: \[(\d+), (\d+)\]", r.stdout.strip())
    out = {"lower": int(line.group(1)), "upper": int(line.group(2))} if line else {"raw": r.stdout.strip()}
    if m:
        out.update({"reduced_n": int(m.group(1)), "bfs_steps": int(m.group(2))})
    elif "Skipping reduction" in r.stderr:
        out["skipped"] = True
    return out


def fixture_reduce():
    """Reduce outcomes (reduced N, BFS steps, shifted bounds) from the reference's log."""
    cases = []
    readme = json.loads((HERE / "readme.json").read_text())["automata"][3]
    inputs = [(readme["n"], readme["k"], None, readme["delta"])]
    inputs += [(n, k, seed, gen.random_dfa(n, k, seed)) for n, k, seed in
               [(80, 2, 1), (100, 2, 2), (100, 3, 3), (128, 2, 4), (150, 2, 5), (200, 2, 6), (200, 3, 7),
                (256, 2, 8)]]
    for n, k, seed, d in inputs:
        r = reference_reduce(REDUCE_ONLY, n, k, d)
        cases.append({"n": n, "k": k, "seed": seed, "delta": d if seed is None else None, "reference": r})
    assert cases[0]["reference"].get("reduced_n") == 90 and cases[0]["reference"]["bfs_steps"] == 8
    write("reduce.json", {"plan": REDUCE_ONLY, "cases": cases})


def fixture_big():
    for n in (320, 384):
        fixture_random(f"random_n{n}.json", n, 2, range(1, 9), {"beam_exact": BEAM_EXACT}, threads=8)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--big", action="store_true")
    ap.add_argument("--only", default="")
    a = ap.parse_args()
    steps = {
        "families": fixture_families,
        "readme": fixture_readme,
        "n48": lambda: fixture_random("random_n48.json", 48, 2, range(1, 65), {"exact_default": EXACT_DEFAULT},
                                      with_trace=True),
        "n200": lambda: fixture_random("random_n200.json", 200, 2, range(1, 17),
                                       {"exact_default": EXACT_DEFAULT, "beam_exact": BEAM_EXACT}, threads=8,
                                       with_trace=True),
        "beam": fixture_beam,
        "batch": fixture_batch,
        "eppstein": fixture_eppstein,
        "brute": fixture_brute,
        "reduce": fixture_reduce,
        "edges": fixture_edges,
        "batchref": fixture_batch_more_checks,
    }
    if a.big:
        steps["big"] = fixture_big
    for name, fn in steps.items():
        if a.only and name not in a.only.split(","):
            continue
        t = time.time()
        fn()
        print(f"{name}: {time.time() - t:.1f}s", flush=True)


if __name__ == "__main__":
    main()
