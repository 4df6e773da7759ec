"""Vectorised CPU restatements of one VMC iteration, used as the timed CPU baseline (test
infrastructure and baseline only, never the product): sr_step for the RBM / TFIM chain
workload and resconv_sr_step for the ResConv / J1-J2 square workload.

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

from . import philox
from .rbm import logcosh


def spd_solve_inplace(T, b):
    """y = T^-1 b for a symmetric positive-definite C-ordered T, by LAPACK potrf/potrs on T's
    own memory (T is overwritten by its factor). T.T is the same buffer in Fortran order and T
    is symmetric, so no copy of the n x n matrix is made: at n = 32768 the matrix alone is
    8.6 GB, and a copying solve runs out of host memory. Same factorisation as the reference's
    jax.scipy.linalg.solve(assume_a="pos") (quantax/optimizer/solver.py:50-62)."""
    from scipy.linalg import lapack
    c, info = lapack.dpotrf(T.T, lower=1, clean=0, overwrite_a=1)
    if info != 0:
        raise np.linalg.LinAlgError(f"potrf info {info}")
    y, info = lapack.dpotrs(c, np.asarray(b, dtype=np.float64), lower=1)
    if info != 0:
        raise np.linalg.LinAlgError(f"potrs info {info}")
    return y


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
    y = spd_solve_inplace(T, eb)
    x = Ob.T @ y
    t5 = time.perf_counter()
    M, N = W.shape
    W = (W - lr * x[:M * N].reshape(M, N)).astype(np.float32).astype(np.float64)
    b = (b - lr * x[M * N:]).astype(np.float32).astype(np.float64)
    if timings is not None:
        timings.update(sweep=t1 - t0, eloc=t2 - t1, obar=t3 - t2, gram=t4 - t3, solve=t5 - t4)
    return W, b, s, float(E.mean())


# ---- ResConv on the J1-J2 square lattice ------------------------------------------------------
def _resconv_forward(p32, spins, L, nblocks, channels, batch=4096):
    """Complex log psi (complex64 numpy) of +-1 configurations, float32 torch on the host
    (quantax/model/conv_nets.py:95-183 with exp_by_scale, the layer sequence of
    oracle.resconv.features; the reference model is float32). Activations are kept
    channels-last, the layout in which the host's convolution runs fastest."""
    import math
    import torch
    import torch.nn.functional as F
    from .resconv import _unflatten, gelu
    cl = torch.channels_last
    ws = [w.contiguous(memory_format=cl) if w.dim() == 4 else w.reshape(1, -1, 1, 1)
          for w in _unflatten(p32, nblocks, channels)]

    def conv(x, w, b):
        y = F.conv2d(F.pad(x, (1, 1, 1, 1), mode="circular"), w)
        return y if b is None else y + b

    out = []
    with torch.no_grad():
        for a in range(0, spins.shape[0], batch):
            x = torch.as_tensor(spins[a:a + batch], dtype=torch.float32).reshape(-1, 1, L, L)
            k = 0
            for blk in range(nblocks):
                res = x
                h = x / math.sqrt(blk + 1)
                h = h / math.sqrt(2.0) if blk == 0 else gelu(h)
                h = gelu(conv(h, ws[k], ws[k + 1])).contiguous(memory_format=cl)
                last = blk == nblocks - 1
                h = conv(h, ws[k + 2], None if last else ws[k + 3])
                k += 3 if last else 4
                if res.shape[1] < h.shape[1]:
                    res = res.repeat(1, h.shape[1] // res.shape[1], 1, 1)
                x = (h + res).contiguous(memory_format=cl)
            x = x / math.sqrt(nblocks + 1)
            n = x.shape[0]
            c2 = channels // 2
            z = torch.complex(x[:, :c2].reshape(n, -1), x[:, c2:].reshape(n, -1))
            m = z.real.max(dim=1, keepdim=True).values
            lse = m.squeeze(1) + torch.log(torch.exp(z - m).sum(dim=1))
            out.append((lse - math.log(z.shape[1])).numpy())
    return np.concatenate(out) if out else np.zeros(0, np.complex64)


def exchange_sweep(forward, s, lp, nbr, nsteps, seed, step0, hop=1, reweight=2.0):
    """SpinExchange Metropolis sweep (common_samplers.py:58-162, metropolis.py:246-322) on the
    shared Philox stream, vectorised over chains; only proposals that change a configuration
    are evaluated (the reference's chunked sweep skips the others too)."""
    s = s.copy()
    lp = lp.copy()
    ns, n = s.shape
    z = nbr.shape[1]
    chains = np.arange(ns)
    for t in range(step0, step0 + nsteps):
        w = philox.draw(seed, chains, np.full(ns, t, dtype=np.uint64), philox.TAG_PROPOSE)
        u = philox.unit_float(w[:, 1])
        mask = s == hop
        r = philox.bounded(w[:, 0], mask.sum(axis=1))
        i = np.argmax(np.cumsum(mask, axis=1) > r[:, None].astype(np.int64), axis=1)
        j = nbr[i, philox.bounded(w[:, 2], z)].astype(np.int64)
        j = np.where(j < 0, i, j)
        changed = s[chains, i] != s[chains, j]
        c = chains[changed]
        if c.size == 0:
            continue
        new = s[c].copy()
        ci, cj = i[c], j[c]
        new[np.arange(c.size), ci], new[np.arange(c.size), cj] = s[c, cj], s[c, ci]
        lp_new = forward(new)
        acc = reweight * (lp_new.real.astype(np.float64) - lp[c].real.astype(np.float64)) > np.log1p(-u[c])
        s[c[acc]] = new[acc]
        lp[c[acc]] = lp_new[acc]
    return s, lp


def eloc_heisenberg(forward, s, lp, bonds, Jb, chunk=512):
    """E_loc of sum_b J_b [s_i s_j + 2 sign_b (s+s- + s-s+)] (Heisenberg with msr signs folded
    into Jb's off-diagonal element, common_operators.py:23-53): the diagonal plus, for every
    antiparallel bond, element * psi(s')/psi(s) with s' the swapped configuration
    (operator/operator.py:510-562)."""
    ns = s.shape[0]
    bi, bj = bonds[:, 0], bonds[:, 1]
    diag = (s[:, bi].astype(np.float64) * s[:, bj] * Jb[:, 0]).sum(axis=1)
    E = diag.astype(np.complex128)
    for a in range(0, ns, chunk):
        blk = s[a:a + chunk]
        anti = blk[:, bi] != blk[:, bj]
        rows, bs = np.nonzero(anti)
        sp = blk[rows].copy()
        k = np.arange(rows.size)
        sp[k, bi[bs]], sp[k, bj[bs]] = blk[rows, bj[bs]], blk[rows, bi[bs]]
        lpc = forward(sp).astype(np.complex128)
        ratio = np.exp(lpc - lp[a + rows].astype(np.complex128))
        np.add.at(E, a + rows, Jb[bs, 1] * ratio)
    return E


def resconv_jacobian(p32, s, L, nblocks, channels, chunk=256):
    """O = d log psi / d params (complex: d Re + i d Im) per sample, the vjp of
    quantax/state/variational.py:424-495, by torch.func over float32 parameters."""
    import torch
    from torch.func import jacrev, vmap
    from .resconv import log_psi_torch

    def f(p, x):
        lp = log_psi_torch(p, x[None], L, nblocks, channels, True)[0]
        return torch.stack([lp.real, lp.imag])

    jf = vmap(jacrev(f), in_dims=(None, 0))
    out = np.empty((s.shape[0], p32.numel()), dtype=np.complex64)
    for a in range(0, s.shape[0], chunk):
        x = torch.as_tensor(s[a:a + chunk], dtype=torch.float32)
        g = jf(p32, x).numpy()
        out[a:a + chunk] = g[:, 0] + 1j * g[:, 1]
    return out


def resconv_sr_step(params, s, lp, L, nblocks, channels, nbr, bonds, Jb, seed, step0, nsteps, ashift=1e-4,
                    lr=1e-2, timings=None):
    """One whole SR iteration of the ResConv workload: sweep, local energies, O, Obar (FP64, the
    [Re; Im] stacking of QNGD.solve for real parameters and a complex psi, sr.py:76-113), T =
    Obar Obar^T, the diagonal-shifted Cholesky solve (minnorm_shift_eig, solver.py:50-62),
    x = Obar^T y and the float32 parameter update. Returns (params, spins, log psi, energy)."""
    import torch
    p32 = torch.as_tensor(np.asarray(params, dtype=np.float32))
    fwd = lambda x: _resconv_forward(p32, x, L, nblocks, channels)
    t0 = time.perf_counter()
    s, lp = exchange_sweep(fwd, s, lp, nbr, nsteps, seed, step0)
    t1 = time.perf_counter()
    E = eloc_heisenberg(fwd, s, lp, bonds, Jb)
    t2 = time.perf_counter()
    O = resconv_jacobian(p32, s, L, nblocks, channels)
    t3 = time.perf_counter()
    ns = s.shape[0]
    A = np.empty((2 * ns, O.shape[1]), dtype=np.float64)
    mean = O.mean(axis=0, dtype=np.complex128)  # no FP64 copy of O (9 GB at 16384 x 34944)
    A[:ns] = (O.real - mean.real) / np.sqrt(ns)
    A[ns:] = (O.imag - mean.imag) / np.sqrt(ns)
    del O
    eb = (E - E.mean()) / np.sqrt(ns)
    b = np.concatenate([eb.real, eb.imag])
    t4 = time.perf_counter()
    T = A @ A.T
    t5 = time.perf_counter()
    T[np.diag_indices_from(T)] += 1e-12 * np.trace(T) + ashift
    y = spd_solve_inplace(T, b)
    x = A.T @ y
    t6 = time.perf_counter()
    params = (np.asarray(params, np.float32) - (lr * x).astype(np.float32)).astype(np.float32)
    if timings is not None:
        timings.update(sweep=t1 - t0, eloc=t2 - t1, jacobian=t3 - t2, obar=t4 - t3, gram=t5 - t4, solve=t6 - t5)
    return params, s, lp, float(E.real.mean())
