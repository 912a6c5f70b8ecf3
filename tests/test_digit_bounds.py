"""The exactness argument of the tensor-core digit products (ozaki.cu), checked on
the CPU against the constants the kernel is compiled with.

A value is scaled to an integer U (|U| <= 2^(8 nd - 1)) and cut into nd balanced
base-256 digits, every one an integer that bf16 holds exactly, the top one in
[-128, 128] and the others in [-128, 127].  The tensor cores accumulate, per
64-deep k chunk and per weight level L = s + t, the products of at most three
digit pairs, two real products per complex part (Ar Xr - Ai Xi, Ar Xi + Ai Xr),
into an FP32 accumulator: exact while every partial sum stays below 2^24.
"""
import os
import re

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tight-binding_gb300", "csrc", "ozaki.cu")


def _const(name):
    text = open(SRC).read()
    m = re.search(r"\b" + name + r"\s*=\s*(\d+)", text)
    assert m, name
    return int(m.group(1))


def digits_of(u, nd):
    """Balanced base-256 digits, most significant first (u = sum d[s] 256^(nd-1-s))."""
    u = np.asarray(u, dtype=np.int64).copy()
    d = np.zeros((nd,) + u.shape, dtype=np.int64)
    for s in range(nd - 1, 0, -1):
        lo = ((u + 128) & 255) - 128
        d[s] = lo
        u = (u - lo) >> 8
    d[0] = u
    return d


def _extremes(nd):
    top = 2 ** (8 * nd - 1)
    rng = np.random.default_rng(11)
    vals = np.concatenate([np.array([0, 1, -1, top, -top, top - 1, -top + 1, 127, -128, 128, -129]),
                           rng.integers(-top, top + 1, size=20000)])
    return vals


def test_digits_reconstruct_and_stay_in_range():
    for nd in (6, 3):   # A digits (refinement), A digits (Hellmann-Feynman) and X digits
        u = _extremes(nd)
        d = digits_of(u, nd)
        back = np.zeros_like(u)
        for s in range(nd):
            back = back * 256 + d[s]
        assert (back == u).all()
        assert (np.abs(d[0]) <= 128).all()
        assert (d[1:] >= -128).all() and (d[1:] <= 127).all()
        # every digit and its negation is an integer bf16 holds exactly (8 significant bits)
        for v in np.unique(np.concatenate([d.ravel(), -d.ravel()])):
            assert abs(int(v)) <= 256


def test_level_sums_fit_fp32_exactly():
    bk = _const("OZ_BK")
    sa, sb = _const("OZ_SA"), _const("OZ_SB")
    pairs_per_level = max(sum(1 for s in range(sa) for t in range(sb) if s + t == lv) for lv in range(sa + sb - 1))
    assert pairs_per_level == 3
    # |digit| <= 128, so every digit product is <= 2^14; a complex part adds two
    # real products per pair
    bound = pairs_per_level * 2 * bk * 2 ** 14
    assert bound < 2 ** 24, bound
    # the fold takes Re and Im straight from the accumulator: same bound
    assert np.log2(bound) < 22.6 + 1e-9


def test_digit_product_is_exact_in_fp32_for_a_chunk():
    """Emulate one chunk of one level with worst-case digits: the FP32 sum in any
    order equals the exact integer."""
    bk = _const("OZ_BK")
    rng = np.random.default_rng(3)
    for _ in range(20):
        a = rng.choice([-128, 127, 128], size=(3, 2, bk))   # 3 pairs, (re, im), k
        x = rng.choice([-128, 127, 128], size=(3, 2, bk))
        exact = int((a[:, 0] * x[:, 0] - a[:, 1] * x[:, 1]).sum())
        terms = np.concatenate([(a[:, 0] * x[:, 0]).ravel(), (-a[:, 1] * x[:, 1]).ravel()]).astype(np.float32)
        for order in (np.arange(terms.size), rng.permutation(terms.size)):
            acc = np.float32(0)
            for v in terms[order]:
                acc = np.float32(acc + v)
            assert int(acc) == exact
