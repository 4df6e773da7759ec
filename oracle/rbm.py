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
