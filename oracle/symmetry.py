"""Symmetry projection in FP64 numpy (test infrastructure only).

Restates, for spin systems on the periodic L x L square:
  * the group of a list of generators with sectors: every product g_1^m1 g_2^m2 ... ordered
    with m1 slowest, character prod_k exp(-2 pi i m_k q_k / M_k) (quantax/symmetry/symmetry.py:11-57);
    real characters +-1 when the default dtype is real (:41-45);
  * products of symmetries (symmetry.py:394-432) and Z2 inversion (:325-347, :383-391);
  * the lattice maps of Translation (translation.py:7-53), Rotation by pi/2 and Flip of axis 0
    about the lattice centre (common_symmetries.py:107-206), written here from coordinates;
  * psi_symm(s) = sum_g w_g psi(T_g s), w_g = chi_0 chi_g / |G| (symmetry.py:349-392), and
    through it the log-derivatives d log psi_symm = sum_g (w_g psi_g / psi_symm) d log psi_g
    (quantax/state/variational.py:424-511);
  * exact diagonalisation inside a symmetry sector (the projector P = sum_g w_g T_g, Hermitian
    for one-dimensional representations), against the reference's sector energies.

Group elements are permutations p with (T_p s)_i = s[p[i]].
"""
from __future__ import annotations

import itertools

import numpy as np


def square_index(L):
    """site index of (x, y) on the L x L lattice, x along axis 0 (row-major)."""
    return np.arange(L * L).reshape(L, L)


def translation(L, dx, dy):
    """T s at site (x, y) = s at (x + dx, y + dy)."""
    idx = square_index(L)
    x, y = np.meshgrid(np.arange(L), np.arange(L), indexing="ij")
    return idx[(x + dx) % L, (y + dy) % L].reshape(-1)


def rotation90(L):
    """Rotation by +pi/2 about the centre: site i takes the spin of the site that the rotation
    carries onto i, (x, y) <- (y, L - 1 - x)."""
    idx = square_index(L)
    x, y = np.meshgrid(np.arange(L), np.arange(L), indexing="ij")
    return idx[y, L - 1 - x].reshape(-1)


def flip0(L):
    """Mirror of axis 0 about the centre: (x, y) <- (L - 1 - x, y)."""
    idx = square_index(L)
    x, y = np.meshgrid(np.arange(L), np.arange(L), indexing="ij")
    return idx[L - 1 - x, y].reshape(-1)


def _power(p, m):
    out = np.arange(p.size)
    for _ in range(m):
        out = out[p]
    return out


def _period(p):
    q, m = p.copy(), 1
    ident = np.arange(p.size)
    while not np.array_equal(q, ident):
        q, m = q[p], m + 1
    return m


def group(generators, sectors, complex_chars=True):
    """(perms, chars) of the group generated by the given permutations, element
    (m_1, m_2, ...) = g_1^m1 composed with g_2^m2 ..., m_1 slowest."""
    periods = [_period(np.asarray(g)) for g in generators]
    perms, chars = [], []
    for ms in itertools.product(*[range(M) for M in periods]):
        p = np.arange(len(generators[0]))
        chi = 1.0 + 0j
        for g, m, M, q in zip(generators, ms, periods, sectors):
            # the product's element (a, b) indexes row a by the power b of the next generator
            p = p[_power(np.asarray(g), m)]
            if complex_chars:
                chi *= np.exp(-2j * np.pi * q * m / M)
            else:
                if (2 * q) % M:
                    raise ValueError("complex characters with a real dtype")
                chi *= (-1.0 if q else 1.0) ** m
        perms.append(p)
        chars.append(chi)
    return np.stack(perms), np.asarray(chars)


def product(a, b):
    """Product of two groups given as (perms, chars)."""
    pa, ca = a
    pb, cb = b
    return pa[:, pb].reshape(-1, pa.shape[1]), np.outer(ca, cb).reshape(-1)


def weights(chars, z2=0):
    c = np.asarray(chars, dtype=np.complex128)
    if z2:
        c = np.concatenate([c, z2 * c])
    return c * c[0] / c.size


def symm_spins(s, perms, z2=0):
    """(ns, nsymm, N): every T_g s, flipped copies after the permutations."""
    s = np.atleast_2d(s)
    out = s[:, perms]
    if z2:
        out = np.concatenate([out, -out], axis=1)
    return out


def log_psi_symm(log_psi_fn, s, perms, chars, z2=0):
    """log sum_g w_g exp(log psi(T_g s)) per configuration (complex)."""
    s = np.atleast_2d(s)
    ss = symm_spins(s, perms, z2)
    ns, ng, n = ss.shape
    lg = np.asarray(log_psi_fn(ss.reshape(-1, n)), dtype=np.complex128).reshape(ns, ng)
    w = weights(chars, z2)
    m = lg.real.max(axis=1, keepdims=True)
    z = (w[None, :] * np.exp(lg - m)).sum(axis=1)
    with np.errstate(divide="ignore"):
        return m[:, 0] + np.log(z.astype(np.complex128))


def jacobian_symm(log_psi_fn, jac_fn, s, perms, chars, z2=0):
    """d log psi_symm / d params = sum_g v_g O(T_g s), v_g = w_g psi_g / psi_symm."""
    s = np.atleast_2d(s)
    ss = symm_spins(s, perms, z2)
    ns, ng, n = ss.shape
    flat = ss.reshape(-1, n)
    lg = np.asarray(log_psi_fn(flat), dtype=np.complex128).reshape(ns, ng)
    O = np.asarray(jac_fn(flat)).reshape(ns, ng, -1)
    lsym = log_psi_symm(log_psi_fn, s, perms, chars, z2)
    v = weights(chars, z2)[None, :] * np.exp(lg - lsym[:, None])
    return np.einsum("sg,sgp->sp", v, O)


def sector_ground_energy(H, basis_states, perms, chars, z2=0, k=1):
    """Lowest eigenvalue of P H P on the sector of the given one-dimensional representation;
    basis_states: (D, N) +-1 configurations indexing H's rows (every T_g s must be in it)."""
    import scipy.sparse.linalg as sla
    D, n = basis_states.shape
    code = lambda st: ((st > 0).astype(np.int64) << np.arange(n)).sum(axis=-1)
    lookup = {int(c): i for i, c in enumerate(code(basis_states))}
    ss = symm_spins(basis_states, perms, z2)  # (D, nsymm, N)
    idx = np.vectorize(lookup.__getitem__)(code(ss))  # (D, nsymm)
    w = weights(chars, z2)

    def P(v):
        return (w[None, :] * v[idx]).sum(axis=1)

    def mv(v):
        return P(H @ P(v))

    op = sla.LinearOperator((D, D), matvec=mv, dtype=np.complex128)
    rng = np.random.default_rng(0)
    v0 = P(rng.normal(size=D) + 0j)
    vals = sla.eigsh(op, k=k, which="SA", v0=v0, tol=1e-12)[0]
    return np.sort(vals)
