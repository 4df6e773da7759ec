"""RBM_Dense in FP64 (test infrastructure only).

Restates quantax/model/shallow_nets.py:35-126 and quantax/nn/activation.py:17-23:
  theta = W s + b                          (eqx Linear, W (M, N), b (M))
  log psi(s) = sum_i log|cosh(theta_i)| (+ a.s with the optional visible bias)
  local update after flipping site k:  theta += 2 W[:, k] s'_k   (shallow_nets.py:87-108)
  O_s = d log psi / d params = [tanh(theta_i) s_j (i-major, W ravel order), tanh(theta_i)
        (+ s_j for the visible bias)]  -- the closed form of the per-sample vjp in
        quantax/state/variational.py:424-495 for a LogArray output.
Parameter order follows jax.flatten_util.ravel_pytree of the Linear layer: weight then
bias (quantax/state/variational.py:241); the visible bias, absent in the reference, is
appended last.
"""
from __future__ import annotations

import numpy as np


def logcosh(x):
    x = np.abs(x)
    return x + np.log1p(np.exp(-2.0 * x)) - np.log(2.0)


class RBM:
    def __init__(self, W, b, a=None):
        self.W = np.asarray(W, dtype=np.float64)
        self.b = np.asarray(b, dtype=np.float64)
        self.a = None if a is None else np.asarray(a, dtype=np.float64)

    @property
    def M(self):
        return self.W.shape[0]

    @property
    def N(self):
        return self.W.shape[1]

    @property
    def nparams(self):
        return self.M * self.N + self.M + (0 if self.a is None else self.N)

    def params(self):
        p = [self.W.ravel(), self.b]
        if self.a is not None:
            p.append(self.a)
        return np.concatenate(p)

    def set_params(self, p):
        M, N = self.M, self.N
        self.W = p[:M * N].reshape(M, N).copy()
        self.b = p[M * N:M * N + M].copy()
        if self.a is not None:
            self.a = p[M * N + M:].copy()

    def theta(self, s):
        return np.asarray(s, dtype=np.float64) @ self.W.T + self.b

    def log_psi(self, s):
        s = np.atleast_2d(np.asarray(s, dtype=np.float64))
        lp = logcosh(self.theta(s)).sum(axis=1)
        if self.a is not None:
            lp = lp + s @ self.a
        return lp

    def jacobian(self, s):
        s = np.atleast_2d(np.asarray(s, dtype=np.float64))
        t = np.tanh(self.theta(s))
        ns = s.shape[0]
        cols = [(t[:, :, None] * s[:, None, :]).reshape(ns, -1), t]
        if self.a is not None:
            cols.append(s)
        return np.concatenate(cols, axis=1)


def init_normal(N, M, std=0.01, seed=0, visible_bias=False):
    """Parameters drawn N(0, std^2) from a numpy generator (the synthetic-workload init)."""
    rng = np.random.default_rng(seed)
    W = rng.normal(0.0, std, (M, N)).astype(np.float32)
    b = rng.normal(0.0, std, M).astype(np.float32)
    a = rng.normal(0.0, std, N).astype(np.float32) if visible_bias else None
    return W, b, a


class RBMConv:
    """RBM_Conv (quantax/model/shallow_nets.py:129-190): theta[c, x] = b_c + sum_d W[c, d]
    s[x + d - lo] over the periodic lattice (lo = (L - 1) // 2 per axis: the circular SAME
    convolution with a lattice-sized kernel, cross-correlation as lax.conv computes it),
    log psi = sum_{c,x} log cosh theta[c, x]. Written with lattice rolls, independently of the
    device's dense expansion. W: (C, L0, L1), b: (C,); a chain is L1 = 1."""

    def __init__(self, W, b):
        self.W = np.asarray(W, dtype=np.float64)
        self.b = np.asarray(b, dtype=np.float64)
        self.C, self.L0, self.L1 = self.W.shape
        self.lo = ((self.L0 - 1) // 2, (self.L1 - 1) // 2)

    def _shifted(self, s):
        """(ns, L0, L1, L0, L1): [..., d0, d1] = s[x + d - lo] as a lattice over x."""
        s = np.asarray(s, dtype=np.float64).reshape(-1, self.L0, self.L1)
        out = np.empty(s.shape + (self.L0, self.L1))
        for d0 in range(self.L0):
            for d1 in range(self.L1):
                out[..., d0, d1] = np.roll(s, (self.lo[0] - d0, self.lo[1] - d1), axis=(1, 2))
        return out

    def theta(self, s):
        sh = self._shifted(s)  # (ns, x0, x1, d0, d1)
        return np.einsum("cde,nxyde->ncxy", self.W, sh) + self.b[None, :, None, None]

    def log_psi(self, s):
        th = self.theta(np.atleast_2d(s))
        return logcosh(th).reshape(th.shape[0], -1).sum(axis=1)

    def jacobian(self, s):
        s = np.atleast_2d(s)
        t = np.tanh(self.theta(s))  # (ns, C, x0, x1)
        sh = self._shifted(s)
        gW = np.einsum("ncxy,nxyde->ncde", t, sh).reshape(s.shape[0], -1)
        gb = t.reshape(t.shape[0], self.C, -1).sum(axis=2)
        return np.concatenate([gW, gb], axis=1)

    def params(self):
        return np.concatenate([self.W.ravel(), self.b])
