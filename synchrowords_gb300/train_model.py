"""Train the learned distance model on the GPU and write its parameters.

    python -m synchrowords_gb300.train_model --out synchrowords_gb300/models/distance_mlp.f32

Training pairs come from the library itself (sw_distance_pairs): for each
random automaton, sets of its dominance-pruned forward BFS layers labelled with
their exact shortest merge length (subset queries against the inverse BFS
layers from the singletons).  Automata: `--automata` random DFAs with n
uniform in [--n-min, --n-max], k = 2, SplitMix64 seeds from --seed.

The target is the merge length itself; `--relative 1` trains on the merge
length minus the mean over its layer instead (the differences a beam ranks
by; measured worse: per-layer rank correlation 0.28 against 0.51 for set
size).  `--rank-weight W` adds a pairwise ranking term within each layer
(sw_mlp_train_ranked): for siblings with merge lengths a < b,
W * log(1 + exp(y_a - y_b)).  A held-out share is scored after training: mean squared error, and
per layer the rank correlation of predictions with the labels beside the
same correlation for set size (the plain beam's key).
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

from . import DEFAULT_MODEL, MLP_PARAMS, Context
from .generate import random_dfa, splitmix64

FEAT, EMB, HID = 16, 64, 128


def init_params(rng: np.random.Generator, label_mean: float) -> np.ndarray:
    # He initialisation; the embeddings start small (sums over up to n
    # states feed the first layer) and the output starts at the label mean
    parts = [rng.normal(0, (2.0 / FEAT) ** 0.5 / 4, FEAT * EMB), np.zeros(EMB),
             rng.normal(0, (2.0 / EMB) ** 0.5, EMB * HID), np.zeros(HID),
             rng.normal(0, (2.0 / HID) ** 0.5, HID * HID), np.zeros(HID),
             rng.normal(0, (1.0 / HID) ** 0.5 / 10, HID), np.array([label_mean])]
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == MLP_PARAMS
    return p


def spearman(a: np.ndarray, b: np.ndarray) -> float:
    ra = np.argsort(np.argsort(a)).astype(np.float64)
    rb = np.argsort(np.argsort(b)).astype(np.float64)
    if ra.std() == 0 or rb.std() == 0:
        return 0.0
    return float(np.corrcoef(ra, rb)[0, 1])


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--automata", type=int, default=2000)
    ap.add_argument("--n-min", type=int, default=64)
    ap.add_argument("--n-max", type=int, default=128)
    ap.add_argument("--per-layer", type=int, default=256)
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--holdout", type=float, default=0.05)
    ap.add_argument("--out", default=str(DEFAULT_MODEL))
    ap.add_argument("--report", default="")
    ap.add_argument("--relative", type=int, default=0, help="train on merge length minus the layer mean")
    ap.add_argument("--rank-weight", type=float, default=0.0,
                    help="add a pairwise ranking term within each BFS layer, with this weight")
    a = ap.parse_args()

    g = splitmix64(a.seed)
    autos = []
    for _ in range(a.automata):
        n = a.n_min + next(g) % (a.n_max - a.n_min + 1)
        autos.append((n, 2, random_dfa(n, 2, next(g) & 0xFFFFFFFF)))
    ctx = Context(0, model=None)
    t0 = time.time()
    data = []
    for n, k, d in autos:
        sets, labels, depths, length = ctx.distance_pairs(d, n, k, per_layer=a.per_layer)
        if len(labels):
            target = labels.copy()
            if a.relative:
                for dep in np.unique(depths):
                    sel = depths == dep
                    target[sel] -= labels[sel].mean()
            data.append(((n, k, d), sets, target, depths))
    t_pairs = time.time() - t0
    hold = max(1, int(len(data) * a.holdout))
    train, test = data[hold:], data[:hold]
    pairs = sum(len(x[2]) for x in train)
    mean = float(np.mean(np.concatenate([x[2] for x in train])))
    params = init_params(np.random.default_rng(a.seed), mean)
    t1 = time.time()
    params, loss = ctx.mlp_train(params, [x[0] for x in train], [x[1] for x in train], [x[2] for x in train],
                                 epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed,
                                 groups_per_automaton=[x[3] for x in train] if a.rank_weight > 0 else None,
                                 rank_weight=a.rank_weight)
    t_train = time.time() - t1
    mse, mse_mean, rho, rho_size = [], [], [], []
    for (n, k, d), sets, target, depths in test:
        y = ctx.mlp_forward(params, d, n, k, sets)
        size = np.array([sum(bin(int(w)).count("1") for w in row) for row in sets], dtype=np.float64)
        mse.append(float(np.mean((y - target) ** 2)))
        mse_mean.append(float(np.mean((mean - target) ** 2)))
        for dep in np.unique(depths):
            sel = depths == dep
            if sel.sum() >= 8 and target[sel].std() > 0:
                rho.append(spearman(y[sel], target[sel]))
                rho_size.append(spearman(size[sel], target[sel]))
    Path(a.out).parent.mkdir(parents=True, exist_ok=True)
    params.astype("<f4").tofile(a.out)
    report = {"automata": len(data), "train_pairs": pairs, "holdout_automata": len(test),
              "pairs_seconds": round(t_pairs, 1), "train_seconds": round(t_train, 1),
              "last_epoch_loss": round(loss, 4), "holdout_mse": round(float(np.mean(mse)), 4),
              "holdout_mse_of_label_mean": round(float(np.mean(mse_mean)), 4),
              "holdout_layer_rank_correlation": round(float(np.mean(rho)), 4),
              "holdout_layer_rank_correlation_of_size": round(float(np.mean(rho_size)), 4),
              "holdout_layers": len(rho), "target_mean": round(mean, 3),
              "config": vars(a)}
    print(json.dumps(report))
    if a.report:
        Path(a.report).write_text(json.dumps(report, indent=1) + "\n")


if __name__ == "__main__":
    main()
