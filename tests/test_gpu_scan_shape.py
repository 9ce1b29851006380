"""The subset check's launch shape (tile rows, warps per block, tiles per
super-tile, grid factor) and its autotuner: every candidate shape gives the
same answers as brute force, for lists in both size classes and for every row
width class the searches use; solves under tuned and non-default shapes keep
the compiled reference's lengths (tests/golden/random_n200.json)."""
import functools
import json
from pathlib import Path

import numpy as np
import pytest

from synchrowords_gb300.generate import random_dfa

pytestmark = pytest.mark.gpu

EXACT = json.dumps({"algorithms": [{"name": "Exact", "config": {}}]})

# (tile_rows, warps, tiles_per_super, grid_factor): the extremes of each knob and the default
SHAPES = [(32, 4, 4, 1), (32, 16, 32, 64), (64, 8, 16, 16), (128, 4, 8, 4), (128, 16, 32, 32), (64, 16, 4, 8),
          (128, 8, 16, 64)]


def smem_ok(words, tile_rows, warps):
    return 8 * words * tile_rows * 2 * warps <= 200 * 1024


def brute(S, C, proper):
    """For every row c of C: some row s of S with s ⊆ c (s ≠ c when proper)."""
    out = []
    for c in C:
        sub = np.all((S & ~c) == 0, axis=1)
        if proper:
            sub &= ~np.all(S == c, axis=1)
        out.append(int(sub.any()))
    return out


@pytest.fixture
def own_ctx(native_lib):
    import synchrowords_gb300 as sw
    c = sw.Context(0)
    yield c
    c.close()


def test_defaults_and_validation(own_ctx):
    import synchrowords_gb300 as sw
    for words in range(1, 9):
        for cls in range(sw.SCAN_SIZE_CLASSES):
            assert own_ctx.get_scan_shape(words, cls) == sw.DEFAULT_SCAN_SHAPE
    bad = [dict(tile_rows=48), dict(warps=3), dict(warps=32), dict(tiles_per_super=64), dict(tiles_per_super=2),
           dict(grid_factor=0), dict(grid_factor=65)]
    for b in bad:
        with pytest.raises(sw.SynchroError):
            own_ctx.set_scan_shape(4, 0, **b)
    with pytest.raises(sw.SynchroError):
        own_ctx.set_scan_shape(8, 1, tile_rows=128, warps=16)  # two tiles per warp: 256 KiB of shared memory
    for words, cls in ((0, 0), (9, 0), (4, 2)):
        with pytest.raises(sw.SynchroError):
            own_ctx.set_scan_shape(words, cls)
    own_ctx.set_scan_shape(3, 1, tile_rows=32, warps=16, tiles_per_super=4, grid_factor=2)
    assert own_ctx.get_scan_shape(3, 1) == {"tile_rows": 32, "warps": 16, "tiles_per_super": 4, "grid_factor": 2}
    assert own_ctx.get_scan_shape(3, 0) == sw.DEFAULT_SCAN_SHAPE


def set_rows(n, state_lists):
    rows = np.zeros((len(state_lists), (n + 63) // 64), dtype=np.uint64)
    for i, qs in enumerate(state_lists):
        for q in qs:
            rows[i, q // 64] |= np.uint64(1) << np.uint64(q % 64)
    return rows


def clustered_case(rng, n, m, q):
    """S: m sets, grouped by 20 clusters of four shared states plus two
    random states each (so tiles of S share states and their AND masks
    prune); C: q sets, half holding one cluster's states plus sparse random
    states (about half of those contain a set of S), half sparse random sets
    (almost none do), then 30 rows of S itself."""
    clusters = [rng.choice(n, 4, replace=False) for _ in range(20)]
    per = m // 20
    S = []
    for j in range(20):
        for _ in range(per if j < 19 else m - 19 * per):
            S.append(set(clusters[j].tolist()) | set(rng.choice(n, 2).tolist()))
    p = min(0.5, np.sqrt(0.7 / per))
    C = []
    for i in range(q):
        extra = set(np.nonzero(rng.random(n) < p)[0].tolist())
        C.append(extra | (set(clusters[rng.integers(20)].tolist()) if i % 2 == 0 else set()))
    return set_rows(n, S), np.concatenate([set_rows(n, C), set_rows(n, S[:: max(1, m // 30)][:30])])


@functools.lru_cache(maxsize=None)
def case_with_answers(n, m):
    S, C = clustered_case(np.random.default_rng(n * 7 + m), n, m, 600)
    return S, C, {False: brute(S, C, False), True: brute(S, C, True)}


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("n", [48, 200, 320, 512])
def test_every_shape_matches_brute_force(own_ctx, shape, n):
    import synchrowords_gb300 as sw
    tr, warps, tps, gf = shape
    words = (n + 63) // 64
    if not smem_ok(words, tr, warps):
        pytest.skip("shape exceeds the shared-memory limit at this width")
    for m, cls in ((3000, 0), (sw.SCAN_LARGE_ROWS + 4000, 1)):
        own_ctx.set_scan_shape(words, cls, tile_rows=tr, warps=warps, tiles_per_super=tps, grid_factor=gf)
        S, C, want = case_with_answers(n, m)
        for proper in (False, True):
            got = own_ctx.subsets_check(n, S, C, proper=proper).tolist()
            assert got == want[proper], (shape, n, m, proper)
            assert 0.1 * len(got) < sum(got) < 0.9 * len(got), (sum(got), len(got))


def _n200():
    g = json.loads((Path(__file__).resolve().parent / "golden" / "random_n200.json").read_text())
    want = [(r["lower"], r["upper"]) for r in g["reference"]["exact_default"]["results"]]
    return [(200, 2, random_dfa(200, 2, s)) for s in g["seeds"]], want


def test_solves_keep_reference_lengths_under_other_shapes(own_ctx):
    autos, want = _n200()
    for shape in [(32, 16, 4, 64), (128, 4, 32, 4)]:
        tr, warps, tps, gf = shape
        for cls in (0, 1):
            own_ctx.set_scan_shape(4, cls, tile_rows=tr, warps=warps, tiles_per_super=tps, grid_factor=gf)
        for (n, k, d), w in zip(autos[:6], want[:6]):
            r = own_ctx.solve(d, n, k, EXACT)
            assert (r.lower, r.upper) == w, shape


def test_autotuner_keeps_a_valid_shape_and_the_answers(own_ctx):
    import synchrowords_gb300 as sw
    autos, want = _n200()
    tuned = own_ctx.autotune_scan(autos[:4], EXACT, reps=1)
    assert tuned and {t["words"] for t in tuned} == {4}, tuned
    for t in tuned:
        assert t["checks"] > 0 and 0 < t["ms_best"] <= t["ms_start"], t
        assert own_ctx.get_scan_shape(t["words"], t["size_class"]) == t["shape"]
        sh = t["shape"]
        assert sh["tile_rows"] in (32, 64, 128) and sh["warps"] in (4, 8, 16)
        assert sh["tiles_per_super"] in (4, 8, 16, 32) and 1 <= sh["grid_factor"] <= 64
    print("tuned scan shapes:", tuned)
    # the batch workers take the context's shapes too
    res = own_ctx.solve_batch(autos, EXACT, workers=4)
    for (n, k, d), r, w in zip(autos, res, want):
        assert (r.lower, r.upper) == w
    with pytest.raises(ValueError):
        own_ctx.autotune_scan([], EXACT)
    assert sw.DEFAULT_SCAN_SHAPE == {"tile_rows": 64, "warps": 8, "tiles_per_super": 16, "grid_factor": 16}
