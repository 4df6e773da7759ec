"""Spin Hamiltonians, local energies and exact diagonalisation (test infrastructure only).

Restates the reference's operator conventions:
  * op lists in QuSpin format [[opstr, [[J, i, j, ...], ...]], ...]
    (quantax/operator/operator.py:187-238);
  * site operators: sigma_x = "x" with strength 2, sigma_z = "z" with strength 2,
    sigma_p = "+", sigma_m = "-" with strength 1 (quantax/operator/site_operator.py:39-132);
  * application to a basis state: "z" multiplies by x/2, "x" halves J and flips,
    "+" / "-" need the site down / up else the element is invalid (NaN)
    (quantax/operator/operator.py:30-78), operators applied right to left (:98-119);
  * Ising(h, J) = -h sum sigma_x - J sum_<ij> sigma_z sigma_z
    (quantax/operator/common_operators.py:56-71);
  * Heisenberg(J, n_neighbor, msr) = sum_n J_n sum_<ij>_n [2 sign (s+s- + s-s+) + szsz],
    sign = -1 on nearest-neighbour bonds when msr (quantax/operator/common_operators.py:23-53);
  * E_loc(s) = sum_diag + sum_{s'} H_ss' psi(s')/psi(s) (quantax/operator/operator.py:510-562).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import lattice


def ising_op_list(n_sites, bonds, h=0.0, J=1.0):
    ops = []
    if h != 0.0:
        ops.append(["x", [[-h * 2.0, i] for i in range(n_sites)]])
    ops.append(["zz", [[-J * 4.0, int(i), int(j)] for i, j in bonds]])
    return ops


def heisenberg_op_list(bond_shells, J=(1.0,), n_neighbor=(1,), msr=False):
    ops = {"+-": [], "-+": [], "zz": []}
    for Jn, order, bonds in zip(J, n_neighbor, bond_shells):
        sign = -1.0 if (msr and order == 1) else 1.0
        for i, j in bonds:
            i, j = int(i), int(j)
            ops["+-"].append([Jn * 2.0 * sign, i, j])
            ops["-+"].append([Jn * 2.0 * sign, i, j])
            ops["zz"].append([Jn * 4.0, i, j])
    return [[k, v] for k, v in ops.items() if v]


def _apply_site(x, op, J, idx):
    """One site operator on a +-1 configuration (quantax/operator/operator.py:30-78)."""
    if op == "I":
        return x, J
    if op == "n":
        return x, (J if x[idx] > 0 else 0.0)
    if op == "z":
        return x, J * x[idx] / 2.0
    if op == "x":
        x = x.copy(); x[idx] *= -1
        return x, J / 2.0
    if op == "+":
        if x[idx] >= 0:
            return x, np.nan
        x = x.copy(); x[idx] = 1
        return x, J
    if op == "-":
        if x[idx] <= 0:
            return x, np.nan
        x = x.copy(); x[idx] = -1
        return x, J
    raise ValueError(op)


def connected(s, op_list):
    """Diagonal value and the list of (s', H_ss') for one configuration s (+-1 int array)."""
    diag = 0.0
    conn = []
    for opstr, terms in op_list:
        is_diag = all(o in ("I", "n", "z") for o in opstr)
        for J, *index in terms:
            x = np.array(s, dtype=np.int8)
            val = float(J)
            for o, i in zip(reversed(opstr), reversed(index)):
                x, val = _apply_site(x, o, val, int(i))
                if val != val:  # NaN: invalid
                    break
            if val != val:
                continue
            if is_diag:
                diag += val
            elif not np.isclose(val, 0.0):
                conn.append((x, val))
    return diag, conn


def local_energy(spins, op_list, log_psi_fn):
    """E_loc for a batch of +-1 configurations; log_psi_fn maps (k, N) -> complex/real (k,)."""
    spins = np.asarray(spins)
    out = np.zeros(spins.shape[0], dtype=np.complex128)
    lp = log_psi_fn(spins)
    for a, s in enumerate(spins):
        diag, conn = connected(s, op_list)
        e = complex(diag)
        if conn:
            sc = np.stack([c[0] for c in conn])
            hv = np.array([c[1] for c in conn])
            lpc = log_psi_fn(sc)
            e += np.sum(hv * np.exp(lpc - lp[a]))
        out[a] = e
    return out


def _apply_site_batch(x, op, J, idx):
    """Vectorised _apply_site over a batch of configurations x (k, N); J (k,)."""
    if op == "I":
        return x, J
    if op == "n":
        return x, np.where(x[:, idx] > 0, J, 0.0)
    if op == "z":
        return x, J * x[:, idx] / 2.0
    x = x.copy()
    if op == "x":
        x[:, idx] *= -1
        return x, J / 2.0
    if op == "+":
        J = np.where(x[:, idx] < 0, J, np.nan)
        x[:, idx] = 1
        return x, J
    if op == "-":
        J = np.where(x[:, idx] > 0, J, np.nan)
        x[:, idx] = -1
        return x, J
    raise ValueError(op)


def sparse_matrix(n_sites, op_list, nup=None):
    """Sparse H in the computational basis (bit i of the index = site i up).

    With nup given, only the fixed-magnetisation sector is built.
    """
    allb = np.arange(1 << n_sites, dtype=np.int64)
    if nup is None:
        states = allb
    else:
        pc = np.zeros_like(allb)
        for i in range(n_sites):
            pc += (allb >> i) & 1
        states = allb[pc == nup]
    lookup = np.full(1 << n_sites, -1, dtype=np.int64)
    lookup[states] = np.arange(len(states))
    bits = ((states[:, None] >> np.arange(n_sites)[None, :]) & 1).astype(np.int8) * 2 - 1
    weights = np.int64(1) << np.arange(n_sites, dtype=np.int64)
    nst = len(states)
    rows, cols, vals = [np.arange(nst)], [np.arange(nst)], []
    diag = np.zeros(nst)
    for opstr, terms in op_list:
        is_diag = all(o in ("I", "n", "z") for o in opstr)
        for J, *index in terms:
            x = bits
            val = np.full(nst, float(J))
            for o, i in zip(reversed(opstr), reversed(index)):
                x, val = _apply_site_batch(x, o, val, int(i))
            ok = ~np.isnan(val)
            if is_diag:
                diag[ok] += val[ok]
                continue
            ok &= ~np.isclose(val, 0.0)
            b = ((x[ok] > 0).astype(np.int64) * weights).sum(axis=1)
            rows.append(np.flatnonzero(ok)); cols.append(lookup[b]); vals.append(val[ok])
    vals = [diag] + vals
    H = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(nst, nst))
    return H, states


def ground_energy(n_sites, op_list, nup=None):
    """ED ground-state energy (the reference's Operator.diagonalize, operator.py:331-359)."""
    H, _ = sparse_matrix(n_sites, op_list, nup)
    if H.shape[0] <= 512:
        return float(np.linalg.eigvalsh(H.toarray())[0])
    w = spla.eigsh(H, k=1, which="SA", tol=1e-12)[0]
    return float(w[0])


def chain_tfim(L, h=1.0, J=1.0):
    bonds = lattice.neighbors((L,), 1)
    return ising_op_list(L, bonds, h, J)


def square_j1j2(L, J2=0.5, msr=True):
    shells = lattice.neighbors((L, L), [1, 2])
    return heisenberg_op_list(shells, (1.0, J2), (1, 2), msr)
