"""Vectorised CPU restatement of one VMC iteration for the RBM / TFIM workload, used as
the timed CPU baseline (test infrastructure and baseline only, never the product).

It follows the reference's dataflow rather than the GPU design:
  * sweep: per proposal, theta += 2 W[:, k] s'_k for every chain and log psi = sum log
    cosh theta (quantax/model/shallow_nets.py:87-108, sampler/metropolis.py:262-322);
  * E_loc: log psi of every single-flip configuration from theta
    (operator/operator.py:510-562 with the RBM ref_forward);
  * O, Obar, T = Obar Obar^T, diagonal-shifted Cholesky solve and x = Obar^T y in FP64
    (state/variational.py:424-511, optimizer/sr.py:76-195, optimizer/solver.py:50-62).
Draws come from oracle.philox with the same stream layout as the GPU path.
"""
from __future__ import annotations

import time

import numpy as np
import scipy.linalg as sla

from . import philox
from .rbm import logcosh


def sweep(W, b, s, nsteps, seed, step0=0, reweight=2.0):
    s = s.astype(np.float64).copy()
    ns, n = s.shape
    th = s @ W.T + b
    lp = logcosh(th).sum(axis=1)
    chains = np.arange(ns)
    for t in range(step0, step0 + nsteps):
        w = philox.draw(seed, chains, np.full(ns, t, dtype=np.uint64), philox.TAG_PROPOSE)
        k = philox.bounded(w[:, 0], n)
        u = philox.unit_float(w[:, 1])
        sk = s[chains, k]
        th_new = th - 2.0 * sk[:, None] * W[:, k].T
        lp_new = logcosh(th_new).sum(axis=1)
        acc = reweight * (lp_new - lp) > np.log1p(-u)
        th[acc] = th_new[acc]
        lp[acc] = lp_new[acc]
        s[chains[acc], k[acc]] *= -1
    return s, th, lp


def eloc_tfim(W, th, s, h=1.0, J=1.0):
    """E_loc for the PBC chain TFIM: -J sum s_i s_i+1 - h sum_k psi(s^k)/psi(s)."""
    diag = -J * np.sum(s * np.roll(s, -1, axis=1), axis=1)
    lp = logcosh(th).sum(axis=1)
    off = np.zeros(s.shape[0])
    for k in range(s.shape[1]):
        lpk = logcosh(th - 2.0 * s[:, k:k + 1] * W[:, k][None, :]).sum(axis=1)
        off += np.exp(lpk - lp)
    return diag - h * off


def sr_step(W, b, s, seed, step0, nsteps, ashift=1e-4, lr=1e-2, timings=None):
    """One SR iteration; returns (new W, new b, spins, energy)."""
    t0 = time.perf_counter()
    s, th, _ = sweep(W, b, s, nsteps, seed, step0)
    t1 = time.perf_counter()
    E = eloc_tfim(W, th, s)
    t2 = time.perf_counter()
    ns = s.shape[0]
    t = np.tanh(th)
    O = np.concatenate([(t[:, :, None] * s[:, None, :]).reshape(ns, -1), t], axis=1)
    Ob = (O - O.mean(axis=0)) / np.sqrt(ns)
    eb = (E - E.mean()) / np.sqrt(ns)
    t3 = time.perf_counter()
    T = Ob @ Ob.T
    t4 = time.perf_counter()
    T[np.diag_indices_from(T)] += 1e-12 * np.trace(T) + ashift
    y = sla.solve(T, eb, assume_a="pos")
    x = Ob.T @ y
    t5 = time.perf_counter()
    M, N = W.shape
    W = (W - lr * x[:M * N].reshape(M, N)).astype(np.float32).astype(np.float64)
    b = (b - lr * x[M * N:]).astype(np.float32).astype(np.float64)
    if timings is not None:
        timings.update(sweep=t1 - t0, eloc=t2 - t1, obar=t3 - t2, gram=t4 - t3, solve=t5 - t4)
    return W, b, s, float(E.mean())
