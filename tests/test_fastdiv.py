"""The batch kernels divide cell indices by box extents with a multiply and a
shift: q = (x * m) >> 40 with m = 2^40 // d + 1 (`fastdiv_magic` in
lambrex_gb300/csrc/batch.cuh).  The identity q == x // d holds for x < 2^23
and d < 2^17, the limits the batch engine enforces per box.  The hardest
numerator for each divisor is the largest x below 2^23 with remainder d - 1;
this test checks it, and a seeded random sample, for every divisor.
"""
import numpy as np

X_LIMIT = 1 << 23
D_LIMIT = 1 << 17


def _check(x, d):
    m = (np.uint64(1) << np.uint64(40)) // d + np.uint64(1)
    q = (x * m) >> np.uint64(40)  # x * m < 2^64 for these ranges
    assert np.array_equal(q, x // d)


def test_worst_case_numerators_all_divisors():
    d = np.arange(1, D_LIMIT, dtype=np.uint64)
    top = np.uint64(X_LIMIT - 1)
    # largest x < 2^23 with x % d == d - 1
    x = (top + np.uint64(1)) // d * d - np.uint64(1)
    x = np.where(x > top, x - d, x)
    assert np.all(x % d == d - np.uint64(1))
    _check(x, d)
    _check(top + np.zeros_like(d), d)


def test_random_numerators():
    rng = np.random.default_rng(7)
    x = rng.integers(0, X_LIMIT, size=2_000_000, dtype=np.uint64)
    d = rng.integers(1, D_LIMIT, size=2_000_000, dtype=np.uint64)
    _check(x, d)


def test_bound_is_tight_enough():
    # with numerators up to 2^26 the identity fails for some divisors near
    # 2^17, which is why the engine rejects larger boxes
    d = np.arange(D_LIMIT // 2, D_LIMIT, dtype=np.uint64)
    x = (np.uint64(1 << 26)) // d * d - np.uint64(1)
    m = (np.uint64(1) << np.uint64(40)) // d + np.uint64(1)
    q = (x * m) >> np.uint64(40)
    assert np.any(q != x // d)
