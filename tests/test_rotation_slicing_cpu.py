"""The arithmetic of the FP64 tensor-core rotation (rotate_tc64_kernel), checked
on the CPU with exact integer arithmetic.

The kernel scales each row of Q (and column of R) by a power of two so that
every value becomes an integer X = round(x 2^(1077 - E)), |X| < 2^55, cuts X
into seven two's-complement bytes (a signed top byte in [-128, 127] and six
unsigned ones), multiplies byte slices on the tensor cores and sums the pairs
with equal s + t in seven FP32 accumulators, then assembles
T = 2^24 (acc0 2^24 + acc1 2^16 + acc2 2^8 + acc3) + acc4 2^16 + acc5 2^8 + acc6
and rounds 2^(E_r + F_c - 2106) T once to FP64. Here the same steps run with
Python integers: the digit decomposition must be exact, accumulators 0..4 must
stay within 2^24 in magnitude for K <= 64 (so FP32 holds them exactly), and the
result must be within 2^-50 (sum |q r| + w max|q| max|r|) of the exact product,
the bound tests/test_gpu_rotation.py holds the kernel to."""
import struct

import numpy as np
import pytest


def _bits(x):
    return struct.unpack("<Q", struct.pack("<d", float(x)))[0]


def _exp(x):
    return (_bits(x) >> 52) & 0x7FF


def _fixed_point(x, emax):
    b = _bits(x)
    e = (b >> 52) & 0x7FF
    if e == 0:
        return 0
    m = (b & ((1 << 52) - 1)) | (1 << 52)
    d = emax - e
    if d <= 2:
        u = m << (2 - d)
    else:
        s = d - 2
        u = 0 if s >= 54 else (m + (1 << (s - 1))) >> s
    return -u if b >> 63 else u


def _digits(X):
    lo, hi = X & 0xFFFFFFFF, X >> 32          # Python >> is arithmetic
    return [hi >> 16, (hi >> 8) & 0xFF, hi & 0xFF, lo >> 24, (lo >> 16) & 0xFF, (lo >> 8) & 0xFF, lo & 0xFF]


def _to_double(T, p):
    """2^p T rounded to the nearest double (ties to even)."""
    if T == 0:
        return 0.0
    neg, u = T < 0, abs(T)
    top = u.bit_length() - 1
    if top > 52:
        sh = top - 52
        mant, rem, half = u >> sh, u & ((1 << sh) - 1), 1 << (sh - 1)
        if rem > half or (rem == half and mant & 1):
            mant += 1
        u = mant << sh
    v = float(u) * 2.0 ** p
    return -v if neg else v


def _rotate_entry(q, r):
    emax = max(_exp(v) for v in q)
    fmax = max(_exp(v) for v in r)
    A = [_digits(_fixed_point(v, emax)) for v in q]
    B = [_digits(_fixed_point(v, fmax)) for v in r]
    for a, v in zip(A, q):     # exact decomposition, top digit signed
        X = _fixed_point(v, emax)
        assert sum(d << (48 - 8 * s) for s, d in enumerate(a)) == X
        assert -128 <= a[0] <= 127 and all(0 <= d <= 255 for d in a[1:])
    acc = [sum(A[j][s] * B[j][d - s] for s in range(d + 1) for j in range(len(q))) for d in range(7)]
    assert all(abs(acc[d]) <= 2 ** 24 for d in range(5)), acc
    hi = (acc[0] << 24) + (acc[1] << 16) + (acc[2] << 8) + acc[3]
    lo = (acc[4] << 16) + (acc[5] << 8) + acc[6]
    return _to_double((hi << 24) + lo, emax + fmax - 2106)


def _check(q, r):
    exact = float(sum(np.longdouble(a) * np.longdouble(b) for a, b in zip(q, r)))
    got = _rotate_entry(q, r)
    scale = float(np.sum(np.abs(q) * np.abs(r)) + len(q) * np.abs(q).max() * np.abs(r).max())
    assert abs(got - exact) <= 2.0 ** -50 * scale, (got, exact, scale)


@pytest.mark.parametrize("seed", range(6))
def test_random_rows_and_columns(seed):
    rng = np.random.default_rng(seed)
    for _ in range(40):
        w = int(rng.integers(1, 65))
        q = rng.standard_normal(w) * np.exp2(rng.integers(-20, 20, size=w))
        r = rng.standard_normal(w) * np.exp2(rng.integers(-6, 6, size=w))
        _check(q, r)


def test_largest_digits_at_full_width():
    # Mantissas of all ones at w = 64: the accumulator bound is tightest here.
    x = 1.0 - 2.0 ** -53
    for sq, sr in ((1, 1), (-1, 1), (1, -1)):
        _check(np.full(64, sq * x), np.full(64, sr * x))
    alt = np.array([x, -x] * 32)
    _check(alt, np.full(64, x))


def test_orthonormal_rotation_columns():
    # The engine's case: rows of an orthonormal basis times an orthogonal R.
    rng = np.random.default_rng(9)
    Q, _ = np.linalg.qr(rng.standard_normal((500, 57)))
    R, _ = np.linalg.qr(rng.standard_normal((57, 57)))
    for i in range(0, 500, 25):
        for c in range(0, 57, 7):
            _check(Q[i], R[:, c])


def test_zero_and_tiny_entries():
    q = np.array([0.0, 1e-300, -3.0, 0.0, 5e-310])   # a subnormal entry counts as zero
    r = np.array([1.0, 2.0, 0.5, -7.0, 1.0])
    _check(q, r)
    assert _rotate_entry(np.zeros(5), r) == 0.0
