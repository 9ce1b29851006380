"""ORACLE — test infrastructure, not product.

Numpy restatement of the learned distance model's forward and backward pass
(the CUDA kernels in synchrowords_gb300/csrc/mlp.cu driven by learn.cu), with
bf16 rounding at the same points: feature rows, weights and every activation
fed to a product are rounded to bf16 (round to nearest even); products
accumulate in fp32.  Only tests import this module, to check the device
forward values and gradients.
"""
from __future__ import annotations

import numpy as np

FEAT, EMB, HID = 16, 64, 128
OFF = {}
_o = 0
for _name, _size in (("phi", FEAT * EMB), ("c", EMB), ("w1", EMB * HID), ("b1", HID), ("w2", HID * HID),
                     ("b2", HID), ("w3", HID), ("b3", 1)):
    OFF[_name] = (_o, _size)
    _o += _size
PARAMS = _o


EXACT = False  # True: no bf16 rounding, float64 throughout (for finite-difference checks)


def bf16(x) -> np.ndarray:
    """Round float32 to bf16 (nearest even), returned as float32."""
    if EXACT:
        return np.asarray(x, dtype=np.float64)
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(p: np.ndarray) -> dict:
    shapes = {"phi": (FEAT, EMB), "c": (EMB,), "w1": (EMB, HID), "b1": (HID,), "w2": (HID, HID), "b2": (HID,),
              "w3": (HID,), "b3": (1,)}
    dt = np.float64 if EXACT else np.float32
    return {k: np.asarray(p[o:o + s], dtype=dt).reshape(shapes[k]) for k, (o, s) in OFF.items()}


def bits(sets_ref8: np.ndarray, n: int) -> np.ndarray:
    """[B, 8] uint64 rows (state q = bit q % 64 of word q / 64) -> [B, n] 0/1 float32."""
    s = np.asarray(sets_ref8, dtype=np.uint64).reshape(-1, 8)
    q = np.arange(n)
    return ((s[:, q // 64] >> (q % 64).astype(np.uint64)) & np.uint64(1)).astype(np.float32)


def forward(p: np.ndarray, feat: np.ndarray, b: np.ndarray):
    P = unpack(p)
    fb = bf16(feat)
    epre = fb @ bf16(P["phi"]) + P["c"]
    e = bf16(np.maximum(epre, 0))
    x = bf16(b @ e)
    h1pre = x @ bf16(P["w1"]) + P["b1"]
    h1 = bf16(np.maximum(h1pre, 0))
    h2pre = h1 @ bf16(P["w2"]) + P["b2"]
    h2 = bf16(np.maximum(h2pre, 0))
    y = h2 @ P["w3"] + P["b3"][0]
    cache = dict(P=P, fb=fb, epre=epre, b=b, x=x, h1pre=h1pre, h1=h1, h2pre=h2pre, h2=h2, y=y)
    return (y if EXACT else y.astype(np.float32)), cache


def backward(cache: dict, t: np.ndarray):
    """Gradient of mean((y - t)^2) as a flat vector, and the loss."""
    P = cache["P"]
    y = cache["y"]
    B = len(y)
    d = y - t
    loss = float(np.mean(d * d))
    dy = 2.0 * d / B if EXACT else (2.0 * d / B).astype(np.float32)
    g = {}
    g["w3"] = cache["h2"].T @ dy
    g["b3"] = np.array([dy.sum()])
    dh2 = np.outer(dy, P["w3"]) * (cache["h2pre"] > 0)
    g["b2"] = dh2.sum(0)
    dh2b = bf16(dh2)
    g["w2"] = cache["h1"].T @ dh2b
    dh1 = (dh2b @ bf16(P["w2"]).T) * (cache["h1pre"] > 0)
    g["b1"] = dh1.sum(0)
    dh1b = bf16(dh1)
    g["w1"] = cache["x"].T @ dh1b
    dx = bf16(dh1b @ bf16(P["w1"]).T)
    de = (cache["b"].T @ dx) * (cache["epre"] > 0)
    g["c"] = de.sum(0)
    g["phi"] = cache["fb"].T @ bf16(de)
    flat = np.zeros(PARAMS, dtype=np.float64 if EXACT else np.float32)
    for k, (o, s) in OFF.items():
        flat[o:o + s] = np.asarray(g[k]).reshape(-1)
    return flat, loss
