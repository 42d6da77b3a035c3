"""Host model of the tensor-core FP64 residual's arithmetic (digit_residual.cu).

The kernel forms A x from eight balanced base-128 digits of each operand,
sums the digit products of weight classes w = p + q <= 7 in FP32 over chunks
of 256 k, folds the class sums into two int64 words and scales the result.
These tests check, with numpy on the host, the facts the kernel relies on:

* the split is exact up to its stated remainder: F = round(a' 2^56) taken
  from the bits of the double, a' = sum_p d_p 128^-(p+1) + r, |r| <= 2^-57,
  |d_p| <= 64 (so every digit is exact in BF16);
* FP32 class sums over 256 k are exact whatever the order of accumulation
  (every partial sum is an integer of magnitude <= 2^23);
* the int64 fold and the final scaling reproduce A x within the bound
  2^-50 n max_k|a_ik| max_k|x_k| stated in the kernel's header, and in
  practice within a small multiple of FP64's own rounding.
"""
import numpy as np
import pytest

PLANES = 8


def _keys(M):
    """Per row: the largest key max(biased exponent, 1) over the non-zero
    entries (0 for a zero row), and the scale exponent key - 1021."""
    b = np.ascontiguousarray(M, dtype=np.float64).view(np.uint64) & np.uint64(0x7FFFFFFFFFFFFFFF)
    be = (b >> np.uint64(52)).astype(np.int64)
    key = np.where(b == 0, 0, np.maximum(be, 1)).max(axis=1)
    return np.where(key == 0, 0, key - 1021).astype(np.int64)


def _fixed(M, e):
    """F = round(v 2^(56 - e)), half away from zero, from the bits of v."""
    b = np.ascontiguousarray(M, dtype=np.float64).view(np.uint64)
    be = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    m = (b & np.uint64((1 << 52) - 1)).astype(np.int64)
    x = np.where(be == 0, -1074, be - 1075)
    m = np.where(be == 0, m, m | (1 << 52))
    sh = x - e[:, None] + 56
    up = m << np.clip(sh, 0, 62)
    k = np.clip(-sh, 1, 63)
    dn = (m + (np.int64(1) << (k - 1))) >> k
    F = np.where(sh >= 0, up, np.where(sh > -64, dn, 0))
    return np.where((b >> np.uint64(63)).astype(bool), -F, F)


def _split(M, e):
    """Eight balanced base-128 digits (d_0 most significant) and F."""
    F = _fixed(M, e)
    d = [None] * PLANES
    G = F.copy()
    for p in range(PLANES - 1, 0, -1):
        r = G & 127
        r = np.where(r >= 64, r - 128, r)
        d[p] = r.astype(np.float64)
        G = (G - r) >> 7
    d[0] = G.astype(np.float64)
    return d, F


def _digit_product(A, x):
    """A x (x one column) the way the kernel forms it."""
    n = A.shape[0]
    ea = _keys(A)
    ex = _keys(x.reshape(1, -1))[0]
    da, _ = _split(A, ea)
    dx, _ = _split(x.reshape(1, -1), np.array([ex]))
    hi = np.zeros(n, dtype=np.int64)
    lo = np.zeros(n, dtype=np.int64)
    for k0 in range(0, n, 256):
        sl = slice(k0, min(n, k0 + 256))
        for w in range(PLANES):
            acc = np.zeros(n, dtype=np.float32)
            for p in range(w + 1):
                q = w - p
                # the products are exact in FP32; accumulate term by term
                prod = (da[p][:, sl] * dx[q][0, sl]).astype(np.float32)
                for j in range(prod.shape[1]):
                    acc = acc + prod[:, j]
            S = acc.astype(np.int64)
            if w < 4:
                hi += S * (1 << (7 * (3 - w)))
            else:
                lo += S * (1 << (7 * (7 - w)))
    e = ea + ex
    yh = hi.astype(np.float64)
    lo = lo + (hi - yh.astype(np.int64)) * (1 << 28)
    return np.ldexp(yh, e - 35) + np.ldexp(lo.astype(np.float64), e - 63)


def test_split_is_exact_up_to_remainder():
    rng = np.random.default_rng(1)
    A = rng.standard_normal((64, 300)) * np.ldexp(1.0, rng.integers(-60, 60, size=(64, 1)))
    A[3] = 0.0
    A[5, ::7] = 1e-300
    A[6, :] = 5e-324 * rng.integers(0, 1000, 300)       # subnormal row
    A[7, 0] = 0.5 - 2.0 ** -54                            # rounds up to the top of the range
    e = _keys(A)
    d, F = _split(A, e)
    sc = np.ldexp(A, -e[:, None])
    assert np.abs(sc).max() < 0.5
    assert np.abs(F).max() < 2 ** 55
    for p in range(PLANES):
        assert np.abs(d[p]).max() <= 64
    rec = sum(d[p].astype(np.int64) * 128 ** (PLANES - 1 - p) for p in range(PLANES))
    assert np.array_equal(rec, F)
    # |a' - F 2^-56| <= 2^-57
    assert np.all(np.abs(sc - np.ldexp(F.astype(np.float64), -56)) <= 2.0 ** -57)


def test_fp32_class_sums_are_exact_at_the_limit():
    # every digit at its extreme: 256 k x 8 pairs x 64 x 64 = 2^23
    prod = np.full(256 * 8, 64.0 * 64.0, dtype=np.float32)
    acc = np.float32(0)
    for v in prod:
        acc = np.float32(acc + v)
    assert int(acc) == 256 * 8 * 4096 == 2 ** 23
    # alternating signs and magnitudes: every order gives the integer sum
    rng = np.random.default_rng(2)
    vals = (rng.integers(-64, 65, 2048) * rng.integers(-64, 65, 2048)).astype(np.float32)
    for _ in range(3):
        rng.shuffle(vals)
        a = np.float32(0)
        for v in vals:
            a = np.float32(a + v)
        assert int(a) == int(vals.astype(np.int64).sum())


@pytest.mark.parametrize("n,spread", [(300, 0), (513, 40)])
def test_digit_product_accuracy(n, spread):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    if spread:
        A *= np.ldexp(1.0, rng.integers(-spread, spread, size=(n, 1)))
    x = rng.standard_normal(n) * np.ldexp(1.0, rng.integers(-20, 20, size=n))
    y = _digit_product(A, x)
    exact = (A.astype(np.longdouble) @ x.astype(np.longdouble)).astype(np.float64)
    Ma = np.abs(A).max(axis=1)
    bound = 2.0 ** -50 * n * Ma * np.abs(x).max()
    err = np.abs(y - exact)
    assert np.all(err <= bound)
    # and about as accurate as an FP64 product
    fp64 = np.abs(A @ x - exact)
    scale = np.abs(A) @ np.abs(x)
    assert err.max() <= max(4 * fp64.max(), 2.0 ** -52 * scale.max())
