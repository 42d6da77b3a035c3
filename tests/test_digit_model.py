"""Host model of the tensor-core FP64 residual's arithmetic (digit_residual.cu).

The kernel forms A x from eight balanced base-128 digits of each operand.  The
digits of A are stored as bytes u = d + 64 and turned back into BF16 digits
in the kernel (a byte permute to 128 + u, then an exact subtraction of 192);
the kernel sums the digit products of weight classes w = p + q <= 7 in two
FP32 accumulators (A planes 0-3 and 4-7) over chunks of 1024 k, folds the
class sums into two int64 words and scales the result.  These tests check, with numpy on the host, the facts the kernel
relies on:

* the split is exact up to its stated remainder: F = round(a' 2^56) taken
  from the bits of the double, a' = sum_p d_p 128^-(p+1) + r, |r| <= 2^-57,
  |d_p| <= 64, and the byte fields of F + C7 are the digits plus 64;
* BF16 0x4300 | u is 128 + u for every byte u in [0, 128], the byte permute
  of the kernel makes the two values of bytes 2j, 2j + 1, and subtracting
  192 gives the digits exactly;
* FP32 class sums over 1024 k, at most four digit pairs per class and
  accumulator, are exact whatever the order of accumulation (every partial
  sum is an integer of magnitude <= 2^24);
* the infinity norm from exact integer row sums of |F| (two words per row)
  matches the row sums of |A| within the rounding of the fixed-point values;
* the int64 fold and the final scaling reproduce A x
  within the bound 2^-50 n max_k|a_ik| max_k|x_k| stated in the kernel's
  header, and in practice within a small multiple of FP64's own rounding.
"""
import numpy as np
import pytest

PLANES = 8
C7 = 0x1020408102040  # 64 in each of the seven low base-128 places


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
    for k0 in range(0, n, 1024):
        sl = slice(k0, min(n, k0 + 1024))
        for w in range(PLANES):
            S = np.zeros(n, dtype=np.int64)
            for planes in (range(0, 4), range(4, 8)):         # the two accumulators
                acc = np.zeros(n, dtype=np.float32)
                for p in planes:
                    if p > w:
                        continue
                    q = w - p
                    # the products are exact in FP32; accumulate term by term
                    prod = (da[p][:, sl] * dx[q][0, sl]).astype(np.float32)
                    for j in range(prod.shape[1]):
                        acc = acc + prod[:, j]
                S += acc.astype(np.int64)
            if w < 4:
                hi += S * (1 << (7 * (3 - w)))
            else:
                lo += S * (1 << (7 * (7 - w)))
    e = ea + ex
    yh = hi.astype(np.float64)
    lo = lo + (hi - yh.astype(np.int64)) * (1 << 28)
    return np.ldexp(yh, e - 35) + np.ldexp(lo.astype(np.float64), e - 63)


def _to_bf16_bits(v):
    """BF16 bit patterns of float64 values that BF16 holds exactly."""
    b = np.asarray(v, dtype=np.float32).view(np.uint32)
    assert np.all(b & 0xFFFF == 0)
    return b >> np.uint32(16)


def _bf16(bits):
    """BF16 bit patterns (uint16) as float64."""
    return (np.asarray(bits, dtype=np.uint32) << np.uint32(16)).view(np.float32).astype(np.float64)


def _byte_perm(x, y, sel):
    """CUDA's __byte_perm(x, y, sel) (default mode) on uint32 arrays."""
    b = [(np.uint64(x) >> np.uint64(8 * i)) & np.uint64(0xFF) for i in range(4)] + \
        [(np.uint64(y) >> np.uint64(8 * i)) & np.uint64(0xFF) for i in range(4)]
    out = np.uint64(0)
    for i in range(4):
        out |= b[(sel >> (4 * i)) & 7] << np.uint64(8 * i)
    return int(out)


def test_bf16_operand_of_a_byte():
    u = np.arange(129, dtype=np.uint32)
    assert np.array_equal(_bf16(0x4300 | u), 128.0 + u)
    rng = np.random.default_rng(3)
    for w in rng.integers(0, 129, size=(50, 4)):
        word = int(w[0] | (w[1] << 8) | (w[2] << 16) | (w[3] << 24))
        o0 = _byte_perm(word, 0x43434343, 0x4140)
        o1 = _byte_perm(word, 0x43434343, 0x4342)
        vals = _bf16([o0 & 0xFFFF, o0 >> 16, o1 & 0xFFFF, o1 >> 16])
        assert np.array_equal(vals, 128.0 + w)          # lower k in the low half
        # minus 192 (BF16 0x4340): the digit u - 64, exact in BF16
        assert _bf16(0x4340) == 192.0
        d = vals - 192.0
        assert np.array_equal(d, w.astype(np.float64) - 64)
        assert np.array_equal(_bf16(_to_bf16_bits(d)), d)


def test_digit_bytes_are_the_fields_of_f_plus_c7():
    rng = np.random.default_rng(4)
    A = rng.standard_normal((16, 200)) * np.ldexp(1.0, rng.integers(-30, 30, size=(16, 1)))
    A[2, 3] = 0.5 - 2.0 ** -54
    e = _keys(A)
    d, F = _split(A, e)
    G = F + C7
    for p in range(1, PLANES):
        assert np.array_equal((G >> (7 * (PLANES - 1 - p))) & 127, d[p].astype(np.int64) + 64)
    assert np.array_equal((G >> 49) + 64, d[0].astype(np.int64) + 64)
    for p in range(PLANES):
        u = d[p] + 64
        assert u.min() >= 0 and u.max() <= 128


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
    # every digit at its extreme: 1024 k x 4 pairs x 64 x 64 = 2^24
    prod = np.full(1024 * 4, 64.0 * 64.0, dtype=np.float32)
    acc = np.float32(0)
    for v in prod:
        acc = np.float32(acc + v)
    assert int(acc) == 1024 * 4 * 64 * 64 == 2 ** 24
    # mixed signs and magnitudes: every order gives the integer sum
    rng = np.random.default_rng(2)
    vals = (rng.integers(-64, 65, 4096) * rng.integers(-64, 65, 4096)).astype(np.float32)
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


@pytest.mark.parametrize("n,spread", [(300, 0), (700, 200)])
def test_norm_from_fixed_point_row_sums(n, spread):
    """The infinity norm the split forms from its fixed-point values: per row,
    sum |F| kept exactly as h 2^28 + l (h = sum |F| >> 28, l = sum of the
    low 28 bits), then h 2^(e - 28) + l 2^(e - 56); within n 2^-55 (the
    rounding of each F) plus a few FP64 roundings of the exact row sums."""
    rng = np.random.default_rng(n + spread)
    A = rng.standard_normal((n, n))
    if spread:
        A *= np.ldexp(1.0, rng.integers(-spread, spread, size=(n, 1)))
    A[n // 4] = 0.0
    e = _keys(A)
    F = _fixed(A, e)
    a = np.abs(F).astype(np.uint64)
    h = (a >> np.uint64(28)).sum(axis=1, dtype=np.uint64)
    lo = (a & np.uint64((1 << 28) - 1)).sum(axis=1, dtype=np.uint64)
    rows = np.ldexp(h.astype(np.float64), e - 28) + np.ldexp(lo.astype(np.float64), e - 56)
    assert rows[n // 4] == 0.0
    exact = np.abs(A).astype(np.longdouble).sum(axis=1)
    assert np.all(np.abs(rows - exact) <= (n * 2.0 ** -55 + 2.0 ** -50) * exact + 1e-300)
    norm = rows.max()
    ref = float(exact.max())
    assert abs(norm - ref) <= (n * 2.0 ** -55 + 2.0 ** -50) * ref
