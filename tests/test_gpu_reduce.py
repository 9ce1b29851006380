"""Reduce on the GPU: reduced state count, BFS steps and shifted bounds against
the reference's own log (tests/golden/reduce.json), and Reduce followed by
Exact against the plain exact length (the oracle) with the word checked on the
original automaton."""
import json
from pathlib import Path

import pytest

import oracle
from synchrowords_gb300.generate import random_dfa

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"

# the settings of the reference's README run (configs/readme_config.json)
README_PLAN = {
    "upper_bound": "1ULL * AUT_N * AUT_N * AUT_N / 6", "threads": 1, "gpu": False,
    "algorithms": [
        {"name": "Brute", "config": {"max_n": "20"}},
        {"name": "Eppstein", "config": {"transition_tables": False, "find_word": True}},
        {"name": "Beam", "config": {"presort": "indeg", "beam_size": "10"}},
        {"name": "Reduce", "config": {"min_n": "80", "list_size_threshold": "AUT_N * 16"}},
        {"name": "Exact", "config": {"dfs_min_list_size": "10000", "bfs_small_list_size": "AUT_N * 16",
                                     "dfs": True, "dfs_shortcut": True, "max_memory_mb": "2 * 1024"}}]}


def cases():
    return json.loads((GOLD / "reduce.json").read_text())["cases"]


def automaton(c):
    return c["delta"] or random_dfa(c["n"], c["k"], c["seed"])


@pytest.mark.parametrize("case", cases(), ids=lambda c: f"n{c['n']}k{c['k']}s{c['seed']}")
def test_reduce_matches_reference_log(ctx, case):
    n, k = case["n"], case["k"]
    r = ctx.solve(automaton(case), n, k, json.dumps({"algorithms": [{"name": "Reduce", "config": {}}]}))
    ref = case["reference"]
    assert (r.lower, r.upper) == (ref["lower"], ref["upper"])
    assert (r.stats["reduced_states"], r.stats["reduce_bfs_steps"]) == (ref["reduced_n"], ref["bfs_steps"])


@pytest.mark.parametrize("case", cases(), ids=lambda c: f"n{c['n']}k{c['k']}s{c['seed']}")
def test_reduce_then_exact_keeps_the_exact_length(ctx, case):
    n, k = case["n"], case["k"]
    d = automaton(case)
    plan = {"algorithms": [{"name": "Reduce", "config": {}}, {"name": "Exact", "config": {}}]}
    r = ctx.solve(d, n, k, json.dumps(plan))
    ref = oracle.exact(d, n, k, oracle.ExactParams(threads=4))
    assert (r.lower, r.upper) == (ref.lower, ref.upper)
    assert r.word is not None and len(r.word) == r.upper
    assert len(oracle.apply_word(d, n, k, r.word)) == 1


def test_readme_run(ctx):
    # data/readme_input.txt with configs/readme_config.json; expected lines of docs/install.md:101-104
    g = json.loads((GOLD / "readme.json").read_text())
    for a, exp in zip(g["automata"], g["expected"]):
        n, k, d = a["n"], a["k"], a["delta"]
        r = ctx.solve(d, n, k, json.dumps(README_PLAN))
        if exp.get("non_synchro"):
            assert r.non_synchro
            continue
        assert (r.lower, r.upper) == (exp["lower"], exp["upper"])
        assert [name for name, _ in r.runs] == ["Brute", "Eppstein", "Beam", "Reduce", "Exact"]
        if r.upper:
            assert len(oracle.apply_word(d, n, k, r.word)) == 1


def test_algorithms_after_reduce_leave_bounds_alone(ctx):
    # Beam, Eppstein, Brute and Reduce refuse the reduced automaton (their
    # "not compatible with inputs after reduction" branches); Exact then decides
    c = cases()[0]
    d = automaton(c)
    plan = {"algorithms": [{"name": "Reduce", "config": {}}, {"name": "Beam", "config": {}},
                           {"name": "Eppstein", "config": {}}, {"name": "Reduce", "config": {}}]}
    r = ctx.solve(d, c["n"], c["k"], json.dumps(plan))
    assert (r.lower, r.upper) == (c["reference"]["lower"], c["reference"]["upper"])
    plan["algorithms"].append({"name": "Exact", "config": {}})
    r = ctx.solve(d, c["n"], c["k"], json.dumps(plan))
    assert r.lower == r.upper == 18


def test_cli_readme_run_and_learned_beam(tmp_path):
    """The `synchro` drop-in on the README input and plan (expected lines of
    docs/install.md:101-104), then a plan with LearnedBeam, which ranks by the
    packaged distance model the program finds beside itself."""
    import subprocess
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    cli = root / "synchrowords_gb300" / "_build" / "synchro"
    g = json.loads((GOLD / "readme.json").read_text())
    (tmp_path / "in.txt").write_text("".join(f"{a['k']} {a['n']}\n" + " ".join(map(str, a["delta"])) + "\n"
                                             for a in g["automata"]))
    (tmp_path / "plan.json").write_text(json.dumps(README_PLAN))
    r = subprocess.run([str(cli), "-f", str(tmp_path / "in.txt"), "-c", str(tmp_path / "plan.json"), "-o",
                        str(tmp_path / "out.txt"), "-q"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = (tmp_path / "out.txt").read_text().splitlines()
    assert lines[1] == "1: NON SYNCHRO"
    for i, exp in enumerate(g["expected"]):
        if "lower" in exp:
            assert lines[i].startswith(f"{i}: [{exp['lower']}, {exp['upper']}] ((Brute, ")
    learned = {"algorithms": [{"name": "LearnedBeam", "config": {}}, {"name": "Exact", "config": {}}]}
    (tmp_path / "learned.json").write_text(json.dumps(learned))
    r = subprocess.run([str(cli), "-f", str(tmp_path / "in.txt"), "-c", str(tmp_path / "learned.json"), "-q",
                        "-o", str(tmp_path / "learned.txt")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert (tmp_path / "learned.txt").read_text().splitlines()[3].startswith("3: [18, 18] ((LearnedBeam, ")
    r = subprocess.run([str(cli), "-f", str(tmp_path / "in.txt"), "-c", str(tmp_path / "learned.json"), "-q",
                        "-m", str(tmp_path / "missing.f32")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 1


def test_cli_continue_resumes_after_the_lines_already_written(tmp_path):
    """`synchro --continue` (app/main.cpp:25-53): the automata whose result
    lines are already in the output file (non-empty lines counted) are
    skipped, and the run appends the rest with their original indices.  The
    `-b` build suffix is accepted (there is no JIT build to name)."""
    import subprocess
    root = Path(__file__).resolve().parents[1]
    cli = root / "synchrowords_gb300" / "_build" / "synchro"
    autos = [(30, 2, random_dfa(30, 2, 500 + i)) for i in range(4)]
    (tmp_path / "in.txt").write_text("".join(f"{k} {n}\n" + " ".join(map(str, d)) + "\n" for n, k, d in autos))
    (tmp_path / "plan.json").write_text(json.dumps({"algorithms": [{"name": "Exact", "config": {}}]}))
    base = [str(cli), "-f", str(tmp_path / "in.txt"), "-c", str(tmp_path / "plan.json")]
    r = subprocess.run(base + ["-o", str(tmp_path / "full.txt"), "-q"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    full = (tmp_path / "full.txt").read_text().splitlines()
    assert len(full) == 4
    for i, (n, k, d) in enumerate(autos):
        o = oracle.exact(d, n, k)
        assert full[i].startswith(f"{i}: [{o.lower}, {o.upper}] ((Exact, ")
    # two results already written, then a blank line (not counted)
    (tmp_path / "out.txt").write_text(full[0] + "\n" + full[1] + "\n\n")
    r = subprocess.run(base + ["-o", str(tmp_path / "out.txt"), "--continue", "-b", "suffix"], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Skipping 2 automata" in r.stdout + r.stderr
    got = [s for s in (tmp_path / "out.txt").read_text().splitlines() if s.strip()]
    assert len(got) == 4
    assert got[:2] == full[:2]
    for i in (2, 3):
        assert got[i].split(" ((")[0] == full[i].split(" ((")[0]  # same index and bounds
        word = [int(x) for x in got[i].split("{")[1].rstrip("}").split()]
        n, k, d = autos[i]
        assert len(oracle.apply_word(d, n, k, word)) == 1  # a reset word (the meeting pair found may differ)
    # every automaton already has its line: nothing is appended
    r = subprocess.run(base + ["-o", str(tmp_path / "out.txt"), "--continue", "-q"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert [s for s in (tmp_path / "out.txt").read_text().splitlines() if s.strip()] == got
