"""Host restatements of the binning kernels' arithmetic shortcuts, checked
against the plain computations they replace on adversarial inputs (CPU
only; the compiled device code itself is covered by the GPU parity tests):

* the footprint test |k - c| <= r decided in FP32 outside a rounding band
  (`AbsWithin`, csrc/mg_internal.cuh) never contradicts the FP64 test;
* the galloping search from a guess (`first_true`) equals bisection for any
  guess, including out-of-range ones;
* the reciprocal quotient with correction (`div_exact`, csrc/mg_bin.cu)
  equals integer division.
"""

import bisect

import numpy as np
import pytest

f32 = np.float32


def abs_within_fast(c, r, k):
    """The FP32 decision of AbsWithin: True / False, or None (FP64 decides)."""
    cf, rf = f32(c), f32(r)
    m = f32(abs(cf) + rf + f32(1.0))
    if not m < f32(1.0e6):
        return None
    tol = f32(f32(4.0e-7) * m)
    d = f32(abs(f32(f32(k) - cf)))
    if d <= f32(rf - tol):
        return True
    if d >= f32(rf + tol):
        return False
    return None


def test_fp32_footprint_decisions_agree_with_fp64():
    rng = np.random.default_rng(11)
    n_fast = 0
    for _ in range(200_000):
        scale = 10.0 ** rng.uniform(-1, 6)
        c = rng.uniform(-scale, scale)
        k = int(np.floor(c)) + int(rng.integers(-3, 4))
        # r near the decision boundary |k - c| most of the time
        e = abs(k - c)
        r = max(0.0, e + rng.choice([0.0, 1e-12, -1e-12, 1e-7, -1e-7, 1e-4, -1e-4, 0.3]) * max(1.0, e))
        fast = abs_within_fast(c, r, k)
        if fast is None:
            continue
        n_fast += 1
        assert fast == (abs(float(k) - c) <= r), (c, r, k)
    assert n_fast > 20_000  # the adversarial draws still reach the FP32 path


def test_fp32_decides_typical_footprint_tests():
    rng = np.random.default_rng(12)
    c = rng.uniform(0, 2048, 20_000)
    r = rng.uniform(0.5, 30, 20_000)
    k = np.floor(c + rng.uniform(-1.2, 1.2, 20_000) * r).astype(int)
    decided = sum(abs_within_fast(ci, ri, ki) is not None for ci, ri, ki in zip(c, r, k))
    assert decided > 0.99 * len(c)


def first_true(n, guess, pred):
    """The device search: smallest k in [0, n] with pred(k) (pred(n) true)."""
    guess = min(max(guess, 0), n)
    if guess == n or pred(guess):
        hi, lo, step = guess, guess - 1, 1
        while lo >= 0 and pred(lo):
            hi = lo
            lo -= step
            step <<= 1
        lo = max(lo, -1)
    else:
        lo, hi, step = guess, guess + 1, 1
        while hi < n and not pred(hi):
            lo = hi
            hi += step
            step <<= 1
        hi = min(hi, n)
    while hi - lo > 1:
        m = lo + ((hi - lo) >> 1)
        if pred(m):
            hi = m
        else:
            lo = m
    return hi


@pytest.mark.parametrize("seed", range(5))
def test_galloping_search_equals_bisection(seed):
    rng = np.random.default_rng(seed)
    for _ in range(2000):
        n = int(rng.integers(1, 600))
        edges = np.sort(rng.uniform(-1e3, 1e3, n + 1))
        if rng.random() < 0.3:  # repeated values
            edges = np.round(edges, 0)
        x = rng.uniform(-1.2e3, 1.2e3)
        want = bisect.bisect_left(list(edges[1:]), x)  # first c with edges[c + 1] >= x
        for guess in (want, want - 1, want + 1, 0, n, -5, n + 7, int(rng.integers(0, n + 1))):
            got = first_true(n, guess, lambda c: edges[c + 1] >= x)
            assert got == want, (n, guess, got, want)


def div_exact(a, b):
    """The device quotient: float reciprocal estimate, corrected."""
    rb = f32(1.0 / b)
    q = int(f32(f32(f32(a) + f32(0.5)) * rb))
    r = a - q * b
    while r < 0:
        q -= 1
        r += b
    while r >= b:
        q += 1
        r -= b
    return q


def test_reciprocal_division_is_exact():
    rng = np.random.default_rng(5)
    a = np.concatenate((rng.integers(0, 1 << 24, 50_000), rng.integers(0, 4096, 50_000)))
    b = np.concatenate((rng.integers(1, 300, 50_000), rng.integers(1, 8, 50_000)))
    for ai, bi in zip(a.tolist(), b.tolist()):
        assert div_exact(ai, bi) == ai // bi
