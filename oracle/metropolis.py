"""Metropolis samplers on the shared Philox stream (test infrastructure only).

Restates quantax/sampler/metropolis.py:246-322 and quantax/sampler/common_samplers.py:
  * LocalFlip.propose: one uniform site per chain is flipped (common_samplers.py:28-33);
  * SpinExchange.propose: a uniform site among those holding the hopping particle
    (+1 when 2 Nup <= N, else -1; common_samplers.py:138-142), a uniform entry of its
    padded neighbour row (-1 means "no move"), and the two spins are swapped
    (common_samplers.py:58-82);
  * Metropolis._update: accept when |psi'/psi|^reweight > 1 - u, and only when the
    configuration changed (metropolis.py:291-322).

Draws come from oracle.philox instead of JAX threefry.  For draw t of chain c the
counter is stream_counter(c, t, TAG_PROPOSE) and the four output words are used as
  w0 -> site choice, w1 -> accept uniform u, w2 -> neighbour choice, w3 unused.
The accept test is evaluated in log space: reweight * (log|psi'| - log|psi|) > log(1 - u).

Each run also records the smallest accept margin |reweight*dlogpsi - log(1-u)| seen,
so a test can tell whether an FP32 device run is expected to take the same decisions.
"""
from __future__ import annotations

import numpy as np

from . import philox


def _popcount_select(mask_row, r):
    idx = np.flatnonzero(mask_row)
    return int(idx[r])


def sweep(log_psi_fn, spins, nsteps, seed, step0=0, reweight=2.0, proposal="flip",
          nbr_table=None, hop=1, record=False):
    """Run nsteps Metropolis proposals on every chain.

    log_psi_fn: (k, N) +-1 -> real log|psi| (float64 array).
    spins: (Ns, N) int8 +-1 (copied).
    Returns (spins, log_psi, stats) with stats = dict(min_margin, accepts, sites).
    """
    s = np.array(spins, dtype=np.int8, copy=True)
    ns, n = s.shape
    lp = np.real(log_psi_fn(s))
    chains = np.arange(ns)
    min_margin = np.inf
    accepts = np.zeros(ns, dtype=np.int64)
    site_log = [] if record else None
    for t in range(step0, step0 + nsteps):
        w = philox.draw(seed, chains, np.full(ns, t, dtype=np.uint64), philox.TAG_PROPOSE)
        u = philox.unit_float(w[:, 1])
        new = s.copy()
        if proposal == "flip":
            k = philox.bounded(w[:, 0], n)
            new[chains, k] *= -1
            changed = np.ones(ns, dtype=bool)
            if record:
                site_log.append(k)
        elif proposal == "exchange":
            z = nbr_table.shape[1]
            changed = np.zeros(ns, dtype=bool)
            ks = np.zeros((ns, 2), dtype=np.int64)
            for c in range(ns):
                mask = s[c] == hop
                cnt = int(mask.sum())
                i = _popcount_select(mask, int(philox.bounded(w[c, 0], cnt)))
                j = int(nbr_table[i, int(philox.bounded(w[c, 2], z))])
                if j < 0:
                    j = i
                ks[c] = (i, j)
                if s[c, i] != s[c, j]:
                    new[c, i], new[c, j] = s[c, j], s[c, i]
                    changed[c] = True
            if record:
                site_log.append(ks)
        else:
            raise ValueError(proposal)
        lp_new = np.real(log_psi_fn(new))
        lhs = reweight * (lp_new - lp)
        rhs = np.log1p(-u)
        margin = np.abs(lhs - rhs)
        if changed.any():
            min_margin = min(min_margin, float(margin[changed].min()))
        acc = (lhs > rhs) & changed
        s[acc] = new[acc]
        lp[acc] = lp_new[acc]
        accepts += acc
    stats = dict(min_margin=min_margin, accepts=accepts, sites=site_log)
    return s, np.real(log_psi_fn(s)), stats


def init_uniform(ns, n, seed):
    """Uniform +-1 configurations: bit j of chain c is bit (j % 32) of word (j // 32) % 4
    of the Philox draw at counter stream_counter(c, j // 128, TAG_INIT)."""
    out = np.empty((ns, n), dtype=np.int8)
    chains = np.arange(ns)
    for blk in range((n + 127) // 128):
        w = philox.draw(seed, chains, np.full(ns, blk, dtype=np.uint64), philox.TAG_INIT)
        for j in range(blk * 128, min(n, blk * 128 + 128)):
            word = w[:, (j // 32) % 4]
            bit = (word >> np.uint32(j % 32)) & np.uint32(1)
            out[:, j] = bit.astype(np.int8) * 2 - 1
    return out


def init_fixed_up(ns, n, nup, seed):
    """Configurations with exactly nup up spins: sites 0..nup-1 up, then a Fisher-Yates
    shuffle (i from n-1 down to 1, j = bounded(w0, i+1) of draw (c, i, TAG_INIT_PERM)).
    Mirrors quantax/utils/basis.py:128-133 (independent row permutations)."""
    out = np.full((ns, n), -1, dtype=np.int8)
    out[:, :nup] = 1
    chains = np.arange(ns)
    for i in range(n - 1, 0, -1):
        w = philox.draw(seed, chains, np.full(ns, i, dtype=np.uint64), philox.TAG_INIT_PERM)
        j = philox.bounded(w[:, 0], i + 1)
        a = out[chains, i].copy()
        out[chains, i] = out[chains, j]
        out[chains, j] = a
    return out


def exact_draws(cdf, ns, seed, step):
    """ExactSampler's draw (quantax/sampler/sampler.py:102-110, jr.choice with p = |psi|^n) on
    the shared Philox stream: sample i of sweep `step` is the first j with cdf[j] > u cdf[-1],
    u the 53-bit uniform of draw (seed, i, step, TAG_EXACT); cdf the inclusive prefix sums."""
    w = philox.draw(seed, np.arange(ns), step, philox.TAG_EXACT)
    u = philox.unit_double(w[:, 0], w[:, 1])
    cdf = np.asarray(cdf, dtype=np.float64)
    return np.searchsorted(cdf, u * cdf[-1], side="right")
