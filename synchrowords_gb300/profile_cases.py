"""Small, single-purpose workloads for kernel profiles (ncu captures).

Each case drives one kernel family through the public API on a case small
enough that an ncu capture of a few launches ends in seconds:

  cluster  16 random binary automata, n = 128, on the cluster launch
           (k_cluster_batch, clusters of 8 CTAs)
  small2   64 random binary automata, n = 100, on the shared-memory batched
           launch (k_small_batch, two-word rows)
  small3   the same at n = 150 (three-word rows)
  n200     one plain Exact solve, n = 200, on the streamed path
           (k_subset_scan, k_bitonic_small, k_expand, ...)
  n320     one Beam(dynamic)+Exact solve (the reference's configs/exact.json
           Beam and Exact entries), n = 320: large subset checks of the
           bounded inverse phase
  gemm     one LearnedBeam(4096) run, n = 200 (the model's k_gemm products)

Usage: python -m synchrowords_gb300.profile_cases <case>
"""
from __future__ import annotations

import json
import sys

EXACT = json.dumps({"algorithms": [{"name": "Exact", "config": {}}]})
BEAM_EXACT = json.dumps({
    "upper_bound": "1ULL * (AUT_N - 1) * (AUT_N - 1) + 1",
    "algorithms": [
        {"name": "Beam", "config": {"presort": "indeg", "dynamic": True,
                                    "min_beam_size": "AUT_N * std::log2(AUT_N)",
                                    "max_beam_size": "AUT_N * AUT_N * std::log2(AUT_N)",
                                    "beam_exact_ratio": 0.01}},
        {"name": "Exact", "config": {"dfs_min_list_size": "8192", "bfs_small_list_size": "AUT_N * AUT_K",
                                     "dfs": True, "dfs_shortcut": True, "max_memory_mb": "12 * 1024"}}]})


def run(case: str) -> None:
    import synchrowords_gb300 as sw
    from synchrowords_gb300.generate import random_dfa
    with sw.Context(0) as c:
        if case == "cluster":
            c.set_batch_tuning(workers=8, batched_limit=-1.0, cluster_size=8, cluster_limit=1e9)
            res = c.solve_batch([(128, 2, random_dfa(128, 2, 10 + s)) for s in range(16)], EXACT)
            print([r.upper for r in res])
        elif case in ("small2", "small3"):
            n = 100 if case == "small2" else 150
            c.set_batch_tuning(workers=8, batched_limit=1024.0, cluster_size=-1)
            res = c.solve_batch([(n, 2, random_dfa(n, 2, 20 + s)) for s in range(64)], EXACT)
            print([r.upper for r in res])
        elif case == "n200":
            print(c.solve(random_dfa(200, 2, 1), 200, 2, EXACT).upper)
        elif case == "n320":
            print(c.solve(random_dfa(320, 2, 1), 320, 2, BEAM_EXACT).upper)
        elif case == "gemm":
            plan = json.dumps({"algorithms": [{"name": "LearnedBeam", "config": {"beam_size": "4096"}}]})
            print(c.solve(random_dfa(200, 2, 5), 200, 2, plan).upper)
        else:
            raise SystemExit(f"unknown case {case!r}; cases: cluster small2 small3 n200 n320 gemm")


if __name__ == "__main__":
    run(sys.argv[1] if len(sys.argv) > 1 else "")
