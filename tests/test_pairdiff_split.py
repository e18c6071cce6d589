"""The split-precision argument of the tensor-core pair chi² (csrc/pairdiff.cu, pairtc.cu),
restated in numpy on the CPU.

Each curve is quantised to integers |q| <= QMAX = 127 (65536 + 256 + 1) and split into three
balanced base-256 digits q = 65536 s0 + 256 s1 + s2, each in [-128, 127] and so exact in
bf16.  The nine digit products of a pair accumulate per diagonal d = i + j (five FP32
accumulators): at most three products of |s| <= 128 per epoch, so over T <= 128 epochs every
partial sum stays below 2^24 and FP32 accumulation is exact, and the dot product
p.q = sum_d 256^(4-d) D_d is recovered exactly.  The GPU tests check the kernels.
"""
import numpy as np
import pytest

QMAX = 127 * (65536 + 256 + 1)


def _cmod(a, m):
    """C's % (remainder with the sign of the dividend), as the kernel computes it."""
    return np.fmod(a, m)


def digits(q):
    """k_pd_quantize's balanced digits (C integer semantics)."""
    q = np.asarray(q, np.int64)
    s2 = _cmod(_cmod(q, 256) + 256 + 128, 256) - 128
    r1 = (q - s2) // 256  # exact: q - s2 is a multiple of 256
    s1 = _cmod(_cmod(r1, 256) + 256 + 128, 256) - 128
    s0 = (r1 - s1) // 256
    return s0, s1, s2


def test_digits_reconstruct_and_stay_in_bf16_range():
    rng = np.random.default_rng(0)
    q = np.concatenate([rng.integers(-QMAX, QMAX + 1, 200000), [QMAX, -QMAX, 0, 1, -1, 127, -128, 128, -129]])
    s0, s1, s2 = digits(q)
    assert np.array_equal(65536 * s0 + 256 * s1 + s2, q)
    for s in (s0, s1, s2):
        assert s.min() >= -128 and s.max() <= 127
        assert np.array_equal(s.astype(np.float32).astype(np.int64), s)  # small integers: exact in bf16 too


@pytest.mark.parametrize("extreme", [False, True])
def test_diagonal_sums_exact_in_fp32_and_dot_product_recovered(extreme):
    T, n = 128, 64
    rng = np.random.default_rng(1 + extreme)
    if extreme:  # the largest magnitudes, all epochs of one sign: the bound's worst case
        a = np.full((n, T), QMAX, np.int64) * rng.choice([-1, 1], (n, 1))
        b = np.full((n, T), QMAX, np.int64) * rng.choice([-1, 1], (n, 1))
    else:
        a = rng.integers(-QMAX, QMAX + 1, (n, T))
        b = rng.integers(-QMAX, QMAX + 1, (n, T))
    da, db = digits(a), digits(b)
    exact = a @ b.T  # int64, no overflow: |sum| <= 128 QMAX^2 < 2^53
    rec = np.zeros_like(exact)
    for d in range(5):
        pairs = [(i, d - i) for i in range(3) if 0 <= d - i <= 2]
        D_int = sum(da[i] @ db[j].T for i, j in pairs)
        # the tensor core's FP32 accumulation, epoch by epoch, of this diagonal's products
        acc = np.zeros((n, n), np.float32)
        for t in range(T):
            prod = sum(np.outer(da[i][:, t], db[j][:, t]) for i, j in pairs).astype(np.float32)
            acc = (acc + prod).astype(np.float32)
            assert np.abs(acc).max() < 2 ** 24
        assert np.array_equal(acc.astype(np.int64), D_int)
        rec += 256 ** (4 - d) * D_int
    assert np.array_equal(rec, exact)
