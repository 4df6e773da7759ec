"""The tensor-core Cholesky's exact update C -= P P^T, restated with numpy integers (test
infrastructure only).

Restates the arithmetic of quantax_gb300/csrc/chol.cu (no counterpart in the reference, which
calls jax.scipy.linalg.solve(assume_a="pos"), quantax/optimizer/solver.py:50-62, an FP64
Cholesky): the digit slicing of the error-free transformation of Ozaki, Ogita, Oishi and
Rump (Numer. Algorithms 59, 2012) with 8 balanced base-128 digits per element, the per-level
integer sums the tensor core accumulates, and the int64 fold of the eight levels.
"""
from __future__ import annotations

import numpy as np

SLICES = 8
FIX_BITS = 56


def slice_rows(P):
    """Row exponents e (max |P_r| < 2^e_r) and digits S (SLICES, m, K) int64 with
    P ~= 2^e sum_t S_t 2^(-7 (t + 1))."""
    P = np.asarray(P, dtype=np.float64)
    mx = np.abs(P).max(axis=1)
    e = np.where(mx > 0, np.frexp(mx)[1], 0).astype(np.int64)
    F = np.rint(np.ldexp(P, (FIX_BITS - e)[:, None])).astype(np.int64)
    S = np.empty((SLICES,) + P.shape, dtype=np.int64)
    for t in range(SLICES - 1, 0, -1):
        d = ((F + 64) & 127) - 64
        S[t] = d
        F = (F - d) >> 7
    S[0] = F
    return e, S


def level_sums(S_a, S_b):
    """I_l = sum_{t + u = l} S_t(a) S_u(b)^T for l < SLICES, exact int64 (what the FP32
    accumulators hold when every partial sum stays below 2^24)."""
    m, n = S_a.shape[1], S_b.shape[1]
    out = np.zeros((SLICES, m, n), dtype=np.int64)
    for t in range(SLICES):
        for u in range(SLICES - t):
            out[t + u] += S_a[t] @ S_b[u].T
    return out


def fold(I):
    """V = sum_l I_l 2^(38 - 7 l) in int64, levels 6 and 7 rounded to 2^-38 (chol.cu
    level_term)."""
    V = np.zeros(I.shape[1:], dtype=np.int64)
    for l in range(SLICES):
        s = 38 - 7 * l
        V += I[l] << s if s >= 0 else (I[l] + (1 << (-s - 1))) >> (-s)
    return V


def update(C, P, Q=None):
    """C - P Q^T (Q = P by default) as the kernel computes it: FP64 of the folded integers times
    2^(e_i + e_j - 52), subtracted in FP64 with one fused multiply-add per element."""
    Q = P if Q is None else Q
    ea, Sa = slice_rows(P)
    eb, Sb = slice_rows(Q)
    V = fold(level_sums(Sa, Sb)).astype(np.float64)
    scale = np.ldexp(1.0, (ea[:, None] + eb[None, :] - 52))
    return np.asarray(C, dtype=np.float64) - V * scale
