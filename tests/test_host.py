"""Host-side tests (no GPU): the C ABI library loads and exports every
declared entry point, config expressions evaluate with C++ semantics (checked
against g++ itself), plans parse like the reference's config classes, the CLI
parses the reference's flags, and the bench contract's CPU pieces work."""
import ctypes
import json
import os
import re
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

import synchrowords_gb300 as sw

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "synchrowords.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*|void\*)\s+\**(sw_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(native_lib):
    names = declared_symbols()
    assert len(names) >= 14
    for name in names:
        assert hasattr(native_lib, name), f"{name} missing from the shared library"


def test_version_and_no_device_error(native_lib):
    assert b"sm_103a" in native_lib.sw_version()
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(sw.SynchroError) as e:
        sw.Context(0)
    assert e.value.code == -4  # SW_ERR_NO_DEVICE: no silent CPU path


def test_batch_entry_points_reject_null_arguments(native_lib):
    """The batch and tuning entry points check their pointers before touching
    a context (so this runs without a GPU) and report through sw_last_error."""
    lib = native_lib
    t = sw._BatchTuning(4, 104.0)
    assert lib.sw_get_batch_tuning(None, ctypes.byref(t)) == -1
    assert lib.sw_set_batch_tuning(None, ctypes.byref(t)) == -1
    assert b"NULL" in lib.sw_last_error()
    assert lib.sw_solve_batch(None, 1, None, None, None, b"{}", None, 0) == -1
    assert lib.sw_autotune_batch(None, 1, None, None, None, b"{}", None, None, 0, None, 0, 1, None, None) == -1
    assert lib.sw_autotune_cluster(None, 1, None, None, None, b"{}", None, None, 0, None, 0, 1, None, None) == -1
    assert lib.sw_batch_last_profile(None, None) == -1
    assert lib.sw_get_scan_shape(None, 4, 0, None) == -1
    assert lib.sw_set_scan_shape(None, 4, 0, None) == -1
    assert lib.sw_autotune_scan(None, 1, None, None, None, None, 1, None, 0, None) == -1
    assert lib.sw_mlp_train_ranked(None, None, 0, None, None, None, None, None, None, None, 0.0, 1, 1, 0.0, 0,
                                   None) == -1
    assert b"NULL" in lib.sw_last_error()


def test_noalloc_rejects_misaligned_buffers_before_any_device_work(native_lib):
    """The allocation-free subset check validates its pointers on the host: a
    misaligned set, check or result buffer is refused with
    SW_ERR_INVALID_ARGUMENT before any CUDA call (so this runs without a GPU;
    the addresses are never dereferenced)."""
    lib = native_lib
    good = 0x10000  # 16-byte aligned, never touched
    for d_sets, d_checks, d_results in [(good + 8, good, good), (good, good + 4, good), (good, good, good + 2)]:
        rc = lib.sw_subsets_check_device_noalloc(200, ctypes.c_void_p(d_sets), 10, ctypes.c_void_p(d_checks), 10, 0,
                                                 ctypes.c_void_p(d_results), None)
        assert rc == -1, rc  # SW_ERR_INVALID_ARGUMENT
        assert b"misaligned" in lib.sw_last_error()
    # 8-byte aligned checks and 4-byte aligned results pass the validation; an
    # oversized set list is still refused first
    rc = lib.sw_subsets_check_device_noalloc(64, ctypes.c_void_p(good), (1 << 20) + 1, ctypes.c_void_p(good + 8), 1, 0,
                                             ctypes.c_void_p(good + 4), None)
    assert rc == -7  # SW_ERR_CAPACITY


def test_batch_buffers_layout():
    """The Python batch wrapper packs the automata back to back and gives
    result i a word buffer of max(4096, 4 n^2) entries inside one array."""
    import numpy as np
    autos = [(3, 2, [1, 2, 0, 0, 2, 1]), (40, 1, list(range(1, 40)) + [0]), (2, 4, [0, 1, 1, 0, 0, 0, 1, 1])]
    ns, ks, deltas, res, words, offs = sw.Context._batch_buffers(autos)
    assert ns.tolist() == [3, 40, 2] and ks.tolist() == [2, 1, 4]
    assert deltas.tolist() == [x for a in autos for x in a[2]]
    caps = [max(4096, 4 * n * n) for n, _, _ in autos]
    assert offs.tolist() == [0, caps[0], caps[0] + caps[1], sum(caps)] and words.size == sum(caps)
    for i, cap in enumerate(caps):
        assert res[i].word_capacity == cap
        assert ctypes.addressof(res[i].word.contents) == words.ctypes.data + 4 * int(offs[i])
    # a result whose word was filled in comes back as that slice
    words[offs[1]: offs[1] + 3] = [7, 8, 9]
    res[1].has_word, res[1].word_len, res[1].mlsw_lower_bound, res[1].mlsw_upper_bound = 1, 3, 3, 3
    out = sw.Context._batch_results(res, words, offs)
    assert out[1].word == [7, 8, 9] and (out[1].lower, out[1].upper) == (3, 3) and out[0].word is None
    with pytest.raises(ValueError):
        sw.Context._batch_buffers([(3, 2, [0, 1, 2])])


EXPRESSIONS = [
    "AUT_N * 16", "AUT_N * std::log2(AUT_N)", "AUT_N * AUT_N * std::log2(AUT_N)", "1ULL * AUT_N * AUT_N * AUT_N / 6",
    "1ULL * (AUT_N - 1) * (AUT_N - 1) + 1", "12 * 1024", "1024 * 2", "AUT_N * AUT_K", "AUT_N * AUT_K * AUT_K * 8",
    "std::log2(AUT_N)", "std::sqrt(AUT_N) * 3", "std::pow(AUT_K, 10)", "AUT_N / 3", "-AUT_N / 3", "AUT_N % 7",
    "(AUT_N < 1000 * 1000)", "AUT_N > 100 ? 10000 : 5000", "AUT_N * AUT_N * AUT_N * AUT_N", "-1", "8192",
    "static_cast<int>(AUT_N * 1.5)", "(unsigned)AUT_N - 1000", "1U - 2", "AUT_N << 4", "std::floor(AUT_N / 7.0)",
    "2147483647 + 1", "0.01", "AUT_N * 0.01 + std::exp(1)", "std::min(AUT_N, 64)", "std::max(AUT_K * 5, 3)",
]


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
@pytest.mark.parametrize("n,k", [(200, 2), (48, 3), (1, 1), (512, 16), (100000, 7)])
def test_expression_evaluator_matches_gxx(native_lib, tmp_path, n, k):
    # The reference compiles plan values as #defines; compile them here too and
    # compare with the library's evaluator (as uint64 and as double).
    src = ["#include <cmath>\n#include <cstdio>\n#include <cstdint>\n#include <algorithm>\n",
           f"#define AUT_N ({n})\n#define AUT_K ({k})\nint main() {{\n"]
    for e in EXPRESSIONS:
        src.append(f'  {{ auto v = ({e}); std::printf("%llu %.17g\\n", (unsigned long long)(uint64_t)v, (double)v); }}\n')
    src.append("  return 0;\n}\n")
    (tmp_path / "e.cpp").write_text("".join(src))
    subprocess.run(["g++", "-std=c++17", "-w", "-fwrapv", str(tmp_path / "e.cpp"), "-o", str(tmp_path / "e")],
                   check=True)
    out = subprocess.run([str(tmp_path / "e")], capture_output=True, text=True, check=True).stdout.split("\n")
    for e, line in zip(EXPRESSIONS, out):
        want_u, want_d = line.split()
        got_u, got_d = sw.eval_expression(e, n, k)
        assert float(want_d) == pytest.approx(got_d, rel=1e-15, abs=0), e
        # uint64 conversion of negative doubles is implementation-defined; skip those
        if not (float(want_d) < 0 and "." in want_d):
            assert int(want_u) == got_u, e


def pair_graph_synchronizing(d, n, k):
    """Every pair of states reaches the diagonal (backward BFS over pairs)."""
    pre = [[[] for _ in range(k)] for _ in range(n)]
    for q in range(n):
        for a in range(k):
            pre[d[q * k + a]][a].append(q)
    seen = {(q, q) for q in range(n)}
    todo = list(seen)
    while todo:
        p, q = todo.pop()
        for a in range(k):
            for x in pre[p][a]:
                for y in pre[q][a]:
                    e = (min(x, y), max(x, y))
                    if e not in seen:
                        seen.add(e)
                        todo.append(e)
    return len(seen) == n * (n + 1) // 2


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_host_synchronization_test_and_seeds(tmp_path):
    """The host-side synchronisation test and backward seeds
    (csrc/automaton.cpp, used before every solve) agree with a plain
    pair-graph BFS and a reachability restatement on random, one-letter and
    permutation automata."""
    import random
    cuda_inc = next((p for p in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda")
                     if p and (Path(p) / "include" / "cuda_runtime.h").exists()), None)
    if cuda_inc is None:
        pytest.skip("CUDA headers not found")
    drv = tmp_path / "sync.cpp"
    drv.write_text('#include <cstdio>\n#include "automaton.hpp"\nint main() {\n  unsigned n, k;\n'
                   '  while (std::scanf("%u %u", &n, &k) == 2) {\n    std::vector<uint32_t> d(n * k);\n'
                   '    for (auto& x : d) std::scanf("%u", &x);\n'
                   '    const sw::Automaton A = sw::make_automaton(d.data(), n, k);\n'
                   '    std::printf("%d", (int)sw::is_synchronizing(A));\n'
                   '    for (uint32_t q : sw::backward_seeds(A)) std::printf(" %u", q);\n'
                   '    std::printf("\\n");\n  }\n}\n')
    csrc = ROOT / "synchrowords_gb300" / "csrc"
    subprocess.run(["g++", "-std=c++17", "-O1", "-w", f"-I{csrc}", f"-I{cuda_inc}/include", str(drv),
                    str(csrc / "automaton.cpp"), "-o", str(tmp_path / "sync")], check=True)
    rng = random.Random(3)
    autos = []
    for _ in range(300):
        n, k = rng.randint(1, 30), rng.randint(1, 3)
        mode = rng.randrange(3)  # 0 random, 1 one permutation letter, 2 all letters permutations
        d = [0] * (n * k)
        for a in range(k):
            perm = list(range(n))
            rng.shuffle(perm)
            for q in range(n):
                d[q * k + a] = perm[q] if mode == 2 or (mode == 1 and a == 0) else rng.randrange(n)
        autos.append((n, k, d))
    text = "".join(f"{n} {k} " + " ".join(map(str, d)) + "\n" for n, k, d in autos)
    out = subprocess.run([str(tmp_path / "sync")], input=text, capture_output=True, text=True, check=True).stdout
    lines = [list(map(int, line.split())) for line in out.strip().split("\n")]
    got = [bool(line[0]) for line in lines]
    want = [pair_graph_synchronizing(d, n, k) for n, k, d in autos]
    assert got == want
    assert any(want) and not all(want)
    # backward seeds (exact.cpp:149-164): states of the sink component with a
    # letter of in-degree > 1; a synchronizing automaton has one sink component
    for (n, k, d), line, sync in zip(autos, lines, want):
        if not sync:
            continue
        reach = []
        for q in range(n):
            seen, todo = {q}, [q]
            while todo:
                p = todo.pop()
                for a in range(k):
                    t = d[p * k + a]
                    if t not in seen:
                        seen.add(t)
                        todo.append(t)
            reach.append(seen)
        sink = [q for q in range(n) if all(q in reach[p] for p in reach[q])]
        indeg = [[0] * k for _ in range(n)]
        for q in range(n):
            for a in range(k):
                indeg[d[q * k + a]][a] += 1
        seeds = [q for q in sink if any(indeg[q][a] > 1 for a in range(k))]
        assert sorted(line[1:]) == seeds, (n, k, d)


def test_expression_errors():
    with pytest.raises(sw.SynchroError):
        sw.eval_expression("AUT_X * 2", 10, 2)
    with pytest.raises(sw.SynchroError):
        sw.eval_expression("(1 + ", 10, 2)


# configs/exact.json of the reference (the plan the C5 numbers are quoted on)
EXACT_JSON = {
    "upper_bound": "1ULL * (AUT_N - 1) * (AUT_N - 1) + 1", "threads": 1, "gpu": False,
    "algorithms": [
        {"name": "Brute", "config": {"max_n": "15"}},
        {"name": "Eppstein", "config": {"transition_tables": False, "find_word": False}},
        {"name": "Beam", "config": {"presort": "indeg", "dynamic": True, "min_beam_size": "AUT_N * std::log2(AUT_N)",
                                    "max_beam_size": "AUT_N * AUT_N * std::log2(AUT_N)",
                                    "beam_exact_ratio": 0.01}},
        {"name": "Exact", "config": {"dfs_min_list_size": "8192", "bfs_small_list_size": "AUT_N * AUT_K",
                                     "dfs": True, "dfs_shortcut": True, "max_memory_mb": "12 * 1024"}}]}


def test_plan_evaluation_matches_reference_defines(native_lib):
    p = sw.plan_from_json(json.dumps(EXACT_JSON), 320, 2)
    assert p["upper_bound"] == 319 * 319 + 1
    beam = p["algorithms"][2]
    # values the reference logs for n = 320 ("min beamsize 2663 max beamsize 852165")
    assert (beam["min_beam_size"], beam["max_beam_size"]) == (2663, 852165)
    assert beam["presort_indeg"] == 1 and beam["dynamic"] == 1
    assert beam["beam_exact_ratio"] == pytest.approx(0.01)
    ex = p["algorithms"][3]
    assert (ex["max_memory_mb"], ex["dfs_min_list_size"], ex["bfs_small_list_size"]) == (12288, 8192, 640)
    assert p["algorithms"][0]["max_n"] == 15
    assert (p["algorithms"][1]["transition_tables"], p["algorithms"][1]["find_word"]) == (0, 0)
    others = sw.plan_from_json(json.dumps({"algorithms": [{"name": "Brute"}, {"name": "Eppstein"},
                                                          {"name": "Reduce"}]}), 100, 3)
    br, ep, rd = others["algorithms"]
    assert br["max_n"] == 20 and (ep["transition_tables"], ep["find_word"]) == (0, 0)
    assert (rd["min_n"], rd["list_size_threshold"]) == (80, 1600)
    d = sw.plan_from_json(json.dumps({"algorithms": [{"name": "Exact", "config": {}}]}), 200, 2)
    assert d["upper_bound"] == 200 ** 3 // 6
    ex = d["algorithms"][0]
    assert (ex["dfs"], ex["dfs_shortcut"], ex["strict_memory_limit"]) == (1, 1, 0)
    assert (ex["max_memory_mb"], ex["dfs_min_list_size"], ex["bfs_small_list_size"]) == (2048, 10000, 3200)


def test_learned_beam_plan_entry(native_lib):
    """LearnedBeam (no reference counterpart): defaults, expressions and the
    three orders parse; the kind is 6."""
    d = sw.plan_from_json(json.dumps({"algorithms": [{"name": "LearnedBeam"}]}), 384, 2)["algorithms"][0]
    assert (d["kind"], d["beam_size"], d["max_iter"], d["order"]) == (6, 4096, -1, 0)
    for order, code in (("model", 0), ("size", 1), ("size_model", 2)):
        cfg = {"beam_size": "AUT_N * 16", "max_iter": "AUT_N", "order": order}
        d = sw.plan_from_json(json.dumps({"algorithms": [{"name": "LearnedBeam", "config": cfg}]}), 320, 2)
        assert (d["algorithms"][0]["beam_size"], d["algorithms"][0]["max_iter"]) == (5120, 320)
        assert d["algorithms"][0]["order"] == code


def test_exact_reductions_key(native_lib):
    """The Exact entry's own "reductions" key (auto by default)."""
    d = sw.plan_from_json(json.dumps({"algorithms": [{"name": "Exact"}]}), 200, 2)["algorithms"][0]
    assert d["reductions"] == 0
    for value, code in (("auto", 0), ("always", 1), ("memory", 2)):
        cfg = {"reductions": value}
        d = sw.plan_from_json(json.dumps({"algorithms": [{"name": "Exact", "config": cfg}]}), 200, 2)
        assert d["algorithms"][0]["reductions"] == code


@pytest.mark.parametrize("bad", [
    '{"algorithms": [{"name": "Exact", "config": {"reductions": "never"}}]}',
    '{"algorithms": [{"name": "Exact", "config": {"reductions": 1}}]}',
    '{"algorithms": []}', '{"algorithms": [{"name": "Nope", "config": {}}]}', '{"threads": 0, "algorithms": '
    '[{"name": "Exact", "config": {}}]}', '{"threads": 65, "algorithms": [{"name": "Exact"}]}',
    '{"algorithms": [{"name": "Beam", "config": {"presort": "outdeg"}}]}', '{"algorithms": [', 'null',
    '{"algorithms": [{"name": "LearnedBeam", "config": {"order": "depth"}}]}',
    '{"algorithms": [{"name": "LearnedBeam", "config": {"order": 1}}]}',
    '{"algorithms": [{"name": "LearnedBeam", "config": {"beam_size": "0"}}]}'])
def test_plan_errors(native_lib, bad):
    with pytest.raises(sw.SynchroError) as e:
        sw.plan_from_json(bad, 10, 2)
    assert e.value.code == -2


def test_read_automata_and_format(tmp_path):
    p = tmp_path / "a.txt"
    p.write_text("2 3\n1 2 0 0 2 2\n4 1\n0 0 0 0\n")
    autos = sw.read_automata(p)
    assert autos == [(3, 2, [1, 2, 0, 0, 2, 2]), (1, 4, [0, 0, 0, 0])]
    r = sw.Result(False, 3, 3, [1, 0, 1], [("Exact", 5)])
    assert sw.format_result(7, r) == "7: [3, 3] ((Exact, 5)) {1 0 1}"
    assert sw.format_result(1, sw.Result(True, 0, 0, None, [])) == "1: NON SYNCHRO"
    (tmp_path / "bad.txt").write_text("2 3\n1 2 0 0 2 9\n")
    with pytest.raises(ValueError):
        sw.read_automata(tmp_path / "bad.txt")


def test_cli_flags(native_lib, tmp_path):
    cli = ROOT / "synchrowords_gb300" / "_build" / "synchro"
    r = subprocess.run([str(cli), "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "--continue" in r.stdout
    r = subprocess.run([str(cli), "-c", "x.json"], capture_output=True, text=True)
    assert r.returncode == 1  # missing -f (app/args.hpp:42-47)
    r = subprocess.run([str(cli), "-f", "a", "-c", "b", "-v", "-q"], capture_output=True, text=True)
    assert r.returncode == 1
    r = subprocess.run([str(cli), "-f", "a", "-c", "b", "--continue"], capture_output=True, text=True)
    assert r.returncode == 1


def test_bench_reference_arm_runs_on_cpu():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup",
                        "0", "--workload", "n48", "--ref-sample", "2"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "ms" and line["higher_is_better"] is False
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0


def _gloo_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    v = bench.barrier_max(10.0 * (rank + 1), world)
    dfas = bench.workload_dfas("n48", rank)
    dist.destroy_process_group()
    q.put((rank, v, dfas[0][2][:8]))


def test_multi_rank_max_and_disjoint_shards():
    import multiprocessing as mp
    import random
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = random.randint(20000, 40000)
    procs = [ctx.Process(target=_gloo_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert [v for _, v, _ in out] == [20.0, 20.0]  # max over ranks
    assert out[0][2] != out[1][2]  # each rank solves its own automata (weak scaling)


def test_bench_scan_tuning_uses_held_out_automata():
    """The bench tunes the subset check's launch shape on automata of the
    workload's shape that no rank's timed workload contains."""
    sys.path.insert(0, str(ROOT))
    import bench
    for name in ("n200", "n48", "n320", "batch4096"):
        for rank in (0, 1):
            timed = {tuple(d) for _, _, d in bench.workload_dfas(name, rank)}
            held = bench.workload_dfas(name, rank, held_out=4)
            assert len(held) == 4
            n, k, _, _, _ = bench.WORKLOADS[name]
            if n:
                assert all((a[0], a[1]) == (n, k) for a in held)
            for other in (0, 1):
                timed_other = {tuple(d) for _, _, d in bench.workload_dfas(name, other)}
                assert not any(tuple(d) in timed_other for _, _, d in held), (name, rank, other)
            assert not any(tuple(d) in timed for _, _, d in held)


def test_scan_shape_rules_on_the_host(native_lib):
    """The subset check's launch-shape rule (what sw_set_scan_shape accepts),
    checked without a device: each knob's allowed values, and two tiles per
    warp within the 200 KiB shared-memory limit."""
    import synchrowords_gb300 as sw
    for words in range(1, 9):
        sw.check_scan_shape(words)  # the default shape fits every width
        for tr in (32, 64, 128):
            for warps in (4, 8, 16):
                fits = 8 * words * tr * 2 * warps <= 200 * 1024
                if fits:
                    sw.check_scan_shape(words, tile_rows=tr, warps=warps, tiles_per_super=32, grid_factor=64)
                else:
                    with pytest.raises(sw.SynchroError):
                        sw.check_scan_shape(words, tile_rows=tr, warps=warps)
    for bad in (dict(tile_rows=48), dict(tile_rows=256), dict(warps=2), dict(warps=32), dict(tiles_per_super=2),
                dict(tiles_per_super=64), dict(grid_factor=0), dict(grid_factor=65)):
        with pytest.raises(sw.SynchroError):
            sw.check_scan_shape(4, **bad)
    for words in (0, 9):
        with pytest.raises(sw.SynchroError):
            sw.check_scan_shape(words)
    assert native_lib.sw_scan_shape_check(4, None) == -1
