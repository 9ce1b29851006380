"""The allocation-free subset check (sw_subsets_check_device_noalloc).

Callers that own the whole device budget through their own allocator, or that
may not allocate while serving, pass their own device buffers; the library
uses only its static scratch array.  This file checks that entry point
against the allocating one (sw_subsets_check) on the same inputs, for two
calls in a row (the second reuses the scratch the first left behind), and
that an oversized set list is refused before any device work.  It is named to
run last so that a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

from bitsets import random_sets, to_rows

pytestmark = pytest.mark.gpu


def device_rows(sets, n):
    """Rows in the device layout: W = ceil(n/64) words, state q at bit 63 - q % 64 of word q / 64."""
    W = max(1, (n + 63) // 64)
    out = np.zeros((len(sets), W), dtype=np.uint64)
    for i, s in enumerate(sets):
        for q in s:
            out[i, q // 64] |= np.uint64(1 << (63 - q % 64))
    return out


def run_noalloc(lib, n, sets, checks, proper):
    import torch
    ds = torch.from_numpy(device_rows(sets, n).view(np.int64)).cuda()
    dc = torch.from_numpy(device_rows(checks, n).view(np.int64)).cuda()
    res = torch.full((len(checks),), 7, dtype=torch.int32, device="cuda")  # not zero: the call must clear it
    stream = torch.cuda.current_stream()
    rc = lib.sw_subsets_check_device_noalloc(n, ds.data_ptr(), len(sets), dc.data_ptr(), len(checks),
                                             int(proper), res.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.sw_last_error().decode()
    torch.cuda.synchronize()
    return res.cpu().numpy().astype(np.uint8).tolist()


def test_noalloc_matches_allocating_entry_point_twice(ctx, native_lib):
    rng = np.random.default_rng(2024)
    cases = []
    # first call: 200 states, plain subsets; second: 96 states, proper subsets,
    # fewer sets, so stale masks from the first call would show if reused
    n1 = 200
    S1 = random_sets(rng, n1, 3000, 0.1) + random_sets(rng, n1, 300, 0.4)
    C1 = random_sets(rng, n1, 2000, 0.75) + S1[:50]
    cases.append((n1, S1, C1, False))
    n2 = 96
    S2 = random_sets(rng, n2, 700, 0.15)
    C2 = random_sets(rng, n2, 900, 0.6) + S2[:30] + [frozenset(range(n2))]
    cases.append((n2, S2, C2, True))
    # third: 320 states (five-word rows, an odd word count per tile)
    n3 = 320
    S3 = random_sets(rng, n3, 1001, 0.08)
    C3 = random_sets(rng, n3, 800, 0.8) + S3[:20]
    cases.append((n3, S3, C3, False))
    # fourth: 150 states (three-word rows, 24 bytes: tiles of 64 rows stay 16-byte aligned)
    n4 = 150
    S4 = random_sets(rng, n4, 1500, 0.1)
    C4 = random_sets(rng, n4, 700, 0.75) + S4[:25]
    cases.append((n4, S4, C4, True))
    for n, S, C, proper in cases:
        want = ctx.subsets_check(n, to_rows(S, n), to_rows(C, n), proper=proper).tolist()
        got = run_noalloc(native_lib, n, S, C, proper)
        assert got == want
        assert 0 < sum(got) < len(got)  # both outcomes occur


def device_to_reference_words(rows: np.ndarray) -> np.ndarray:
    """Bit-reverse every 64-bit word: device layout (state q at bit 63 - q % 64)
    to the reference layout (state q at bit q % 64)."""
    rev8 = np.array([int(f"{b:08b}"[::-1], 2) for b in range(256)], dtype=np.uint8)
    b = np.ascontiguousarray(rows, dtype=np.uint64).view(np.uint8).reshape(-1, 8)
    return rev8[b[:, ::-1]].copy().view(np.uint64).reshape(rows.shape)


def test_noalloc_at_the_maximum_set_count(ctx, native_lib):
    """Exactly SW_NOALLOC_MAX_SETS sets of 512 states (eight-word rows): the
    tile and super-tile masks then fill the static scratch to its last word,
    so an off-by-one in its sizing would show here.  Checked against the
    allocating entry point on two calls in a row, and on a sample against a
    numpy restatement."""
    import torch
    n, W, m = 512, 8, 1 << 20
    rng = np.random.default_rng(7)
    # sets of (at most) 4 random states; a check of density d contains one
    # with probability about d^4 per set, so at d = 0.01 .. 0.05 over 2^20
    # sets both outcomes occur
    S = np.zeros((m, W), dtype=np.uint64)
    pos = rng.integers(0, n, size=(m, 4))
    rows = np.repeat(np.arange(m), 4)
    np.bitwise_or.at(S, (rows, (pos // 64).ravel()), np.uint64(1) << (63 - pos % 64).ravel().astype(np.uint64))
    dens = np.repeat([0.01, 0.02, 0.03, 0.04, 0.05, 0.3], 400)
    bits = rng.random((len(dens), n)) < dens[:, None]
    C = np.packbits(bits.reshape(-1, W, 64), axis=2, bitorder="big").view(">u8").reshape(-1, W).astype(np.uint64)
    C = np.concatenate([C, S[rng.integers(0, m, size=48)], S[-16:]])  # the last tile's rows are found too
    want = ctx.subsets_check(n, device_to_reference_words(S), device_to_reference_words(C), proper=False).tolist()
    ds = torch.from_numpy(S.view(np.int64)).cuda()
    dc = torch.from_numpy(C.view(np.int64)).cuda()
    for _ in range(2):
        res = torch.full((len(C),), 7, dtype=torch.int32, device="cuda")
        stream = torch.cuda.current_stream()
        rc = native_lib.sw_subsets_check_device_noalloc(n, ds.data_ptr(), m, dc.data_ptr(), len(C), 0,
                                                        res.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, native_lib.sw_last_error().decode()
        torch.cuda.synchronize()
        got = res.cpu().numpy().astype(np.uint8).tolist()
        assert got == want
    assert 0 < sum(got) < len(got)
    assert all(got[-64:])  # the copied sets are always found
    for i in rng.integers(0, len(C), size=12).tolist():
        hit = bool(np.any(np.all((S & ~C[i]) == 0, axis=1)))
        assert got[i] == int(hit), i


def test_noalloc_rejects_oversized_set_list(native_lib):
    import torch
    dummy = torch.zeros(8, dtype=torch.int64, device="cuda")
    res = torch.zeros(1, dtype=torch.int32, device="cuda")
    too_many = (1 << 20) + 1
    rc = native_lib.sw_subsets_check_device_noalloc(64, dummy.data_ptr(), too_many, dummy.data_ptr(), 1, 0,
                                                    res.data_ptr(), None)
    assert rc == -7  # SW_ERR_CAPACITY, refused before touching the buffers
    assert b"SW_NOALLOC_MAX_SETS" in native_lib.sw_last_error()
