"""Uneven batch of 4096 random automata, n ~ U[32,160], k ~ U{2,3}, solved
through sw_solve_batch (batched launch plus worker streams); every length equals the
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
    non_sync = set(GOLD["non_synchronizing_indices"])
    for i, ((n, k, d), r, L) in enumerate(zip(autos, res, GOLD["lengths"])):
        if i in non_sync:
            assert r.non_synchro, i
            continue
        assert (r.lower, r.upper) == (L, L), (i, n, k, r.lower, r.upper, L)
        assert r.word is not None and len(r.word) == L
        assert len(oracle.apply_word(d, n, k, r.word)) == 1, i
