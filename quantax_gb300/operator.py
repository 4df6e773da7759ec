"""Spin operators: QuSpin-format op lists, algebra, compilation to device tables, local
energies and (small-system) exact diagonalisation.

Mirrors quantax/operator/operator.py:187-595, site_operator.py:8-132 and
common_operators.py:23-71. The op list is compiled once into the qgx_operator_t tables
(diagonal constant / z / zz terms, one-site and two-site flips with their matrix
element for every local spin state); the local-energy kernels then generate the
connected configurations in-kernel instead of materialising them.
"""
from __future__ import annotations

import copy
import ctypes as C
from numbers import Number
from typing import Sequence, Union

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla
import torch

from . import _lib
from .global_defs import get_sites, device


def _apply_site(s: int, op: str, val):
    """One site operator on local spin s (+1/-1): returns (new s, new value or None).

    Same conventions as quantax/operator/operator.py:30-78 for spins.
    """
    if op == "I":
        return s, val
    if op == "n":
        return s, (val if s > 0 else 0.0)
    if op == "z":
        return s, val * s / 2.0
    if op == "x":
        return -s, val / 2.0
    if op == "+":
        return (1, val) if s < 0 else (s, None)
    if op == "-":
        return (-1, val) if s > 0 else (s, None)
    if op == "y":
        raise NotImplementedError("sigma_y needs complex matrix elements, not supported by the qgx tables")
    raise ValueError(f"unknown operator {op!r}")


class CompiledOperator:
    """Device tables of one operator (kept alive with the ctypes struct)."""

    def __init__(self, c0, z, zz, f1, f2):
        dev = device()
        self.c0 = float(c0)
        self._keep = []

        def t(a, dt):
            x = torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
            self._keep.append(x)
            return x

        zi = sorted(z)
        self.z_i = t(np.array(zi, np.int32).reshape(-1), torch.int32)
        self.z_J = t(np.array([z[k] for k in zi], np.float64).reshape(-1), torch.float64)
        zzk = sorted(zz)
        self.zz_ij = t(np.array(zzk, np.int32).reshape(-1), torch.int32)
        self.zz_J = t(np.array([zz[k] for k in zzk], np.float64).reshape(-1), torch.float64)
        f1k = sorted(f1)
        self.f1_i = t(np.array(f1k, np.int32).reshape(-1), torch.int32)
        self.f1_J = t(np.array([f1[k] for k in f1k], np.float64).reshape(-1), torch.float64)
        f2k = sorted(f2)
        self.f2_ij = t(np.array(f2k, np.int32).reshape(-1), torch.int32)
        self.f2_J = t(np.array([f2[k] for k in f2k], np.float64).reshape(-1), torch.float64)
        self.host = dict(c0=c0, z=z, zz=zz, f1=f1, f2=f2)
        p = lambda x: C.c_void_p(x.data_ptr()) if x.numel() else None
        self.struct = _lib.Operator(self.c0, len(zi), p(self.z_i), p(self.z_J), len(zzk), p(self.zz_ij),
                                    p(self.zz_J), len(f1k), p(self.f1_i), p(self.f1_J), len(f2k),
                                    p(self.f2_ij), p(self.f2_J))

    @property
    def max_site(self) -> int:
        h = self.host
        sites = list(h["z"]) + [i for ij in h["zz"] for i in ij] + list(h["f1"]) + [i for ij in h["f2"] for i in ij]
        return max(sites) if sites else -1

    @property
    def max_flips(self) -> int:
        return 2 if len(self.host["f2"]) else (1 if len(self.host["f1"]) else 0)


def compile_op_list(op_list):
    """Classify every term by its action on the local states of its sites.

    Returns host dicts (c0, z{i:J}, zz{(i,j):J}, f1{i:[J(s_i=-1), J(s_i=+1)]},
    f2{(i,j): [J(--), J(-+), J(+-), J(++)]}) with i < j.
    """
    c0 = 0.0
    z, zz, f1, f2 = {}, {}, {}, {}
    for opstr, terms in op_list:
        for J, *index in terms:
            index = [int(i) for i in index]
            if len(index) != len(opstr):
                raise ValueError(f"operator {opstr} needs {len(opstr)} indices")
            sites = sorted(set(index))
            if len(sites) > 2:
                raise NotImplementedError("operator terms on more than two sites are not supported")
            table = {}
            for bits in range(1 << len(sites)):
                loc = {s: (1 if (bits >> k) & 1 else -1) for k, s in enumerate(sites)}
                state = dict(loc)
                val = complex(J) if isinstance(J, complex) else float(J)
                for o, i in zip(reversed(opstr), reversed(index)):
                    state[i], val = _apply_site(state[i], o, val)
                    if val is None:
                        break
                if val is None or val == 0:
                    continue
                if isinstance(val, complex):
                    if val.imag != 0:
                        raise NotImplementedError("complex matrix elements are not supported")
                    val = val.real
                table[tuple(loc[s] for s in sites)] = (tuple(state[s] for s in sites), val)
            flipped = {tuple(i for i, (a, b) in enumerate(zip(k, v[0])) if a != b) for k, v in table.items()}
            if all(len(f) == 0 for f in flipped):
                # diagonal function of <= 2 spins: a + b s_i (+ c s_j + d s_i s_j)
                vals = {k: v[1] for k, v in table.items()}
                if len(sites) == 0:
                    c0 += float(J)
                    continue
                if len(sites) == 1:
                    p, m = vals.get((1,), 0.0), vals.get((-1,), 0.0)
                    c0 += (p + m) / 2
                    z[sites[0]] = z.get(sites[0], 0.0) + (p - m) / 2
                else:
                    f = lambda a, b: vals.get((a, b), 0.0)
                    c0 += (f(1, 1) + f(1, -1) + f(-1, 1) + f(-1, -1)) / 4
                    bi = (f(1, 1) + f(1, -1) - f(-1, 1) - f(-1, -1)) / 4
                    bj = (f(1, 1) - f(1, -1) + f(-1, 1) - f(-1, -1)) / 4
                    d = (f(1, 1) - f(1, -1) - f(-1, 1) + f(-1, -1)) / 4
                    z[sites[0]] = z.get(sites[0], 0.0) + bi
                    z[sites[1]] = z.get(sites[1], 0.0) + bj
                    zz[tuple(sites)] = zz.get(tuple(sites), 0.0) + d
                continue
            if len(flipped) != 1:
                raise NotImplementedError("operator term with a state-dependent set of flipped spins")
            moved = [sites[k] for k in next(iter(flipped))]
            if len(moved) == 1:
                i = moved[0]
                k = sites.index(i)
                by_si = {}
                for loc, (_, val) in table.items():
                    by_si.setdefault(loc[k], set()).add(val)
                    # with a second (diagonal) site the element must not depend on it
                if any(len(v) > 1 for v in by_si.values()) or (len(sites) == 2 and any(
                        len([l for l in table if l[k] == si]) == 1 for si in by_si)):
                    raise NotImplementedError("flip elements conditioned on another spin are not supported")
                e = f1.setdefault(i, [0.0, 0.0])
                for si, vals in by_si.items():
                    e[1 if si > 0 else 0] += next(iter(vals))
            else:
                e = f2.setdefault((sites[0], sites[1]), [0.0, 0.0, 0.0, 0.0])
                for loc, (_, val) in table.items():
                    e[2 * (loc[0] > 0) + (loc[1] > 0)] += val
    return c0, z, zz, f1, f2


class Operator:
    """Quantum operator given as a QuSpin-format op list (operator.py:187-238)."""

    def __init__(self, op_list: list):
        self._op_list = op_list
        self._compiled = None
        self._connectivity = None

    @property
    def op_list(self) -> list:
        return self._op_list

    def compiled(self) -> CompiledOperator:
        if self._compiled is None:
            self._compiled = CompiledOperator(*compile_op_list(self._op_list))
        return self._compiled

    # ---- algebra (operator.py:384-505) ---------------------------------------------------
    def __add__(self, other):
        if isinstance(other, Number):
            if not np.isclose(other, 0.0):
                raise ValueError("Constant shift is not implemented for Operator.")
            return self
        if isinstance(other, Operator):
            op_list = copy.deepcopy(self.op_list)
            names = tuple(op for op, _ in op_list)
            for opstr2, inter in other.op_list:
                if opstr2 in names:
                    op_list[names.index(opstr2)][1] += copy.deepcopy(inter)
                else:
                    op_list.append([opstr2, copy.deepcopy(inter)])
            return Operator(op_list)
        return NotImplemented

    def __radd__(self, other):
        if isinstance(other, Number):
            return self + other
        return NotImplemented

    def __sub__(self, other):
        if isinstance(other, Operator):
            return self + (-other)
        return self + other

    def __rsub__(self, other):
        return (-self) + other

    def __mul__(self, other):
        if isinstance(other, Number):
            op_list = copy.deepcopy(self.op_list)
            for _, inter in op_list:
                for term in inter:
                    term[0] *= other
            return Operator(op_list)
        return NotImplemented

    __rmul__ = __mul__

    def __neg__(self):
        return (-1) * self

    def __truediv__(self, other):
        return self * (1 / other)

    def __matmul__(self, other):
        if isinstance(other, Operator):
            op_list = []
            for s1, i1 in self.op_list:
                for s2, i2 in other.op_list:
                    op = [s1 + s2, []]
                    for J1, *a in i1:
                        for J2, *b in i2:
                            op[1].append([J1 * J2, *a, *b])
                    op_list.append(op)
            return Operator(op_list)
        return NotImplemented

    @property
    def H(self):
        op_list = copy.deepcopy(self.op_list)
        for i, (opstr, inter) in enumerate(op_list):
            op_list[i][0] = opstr.translate(str.maketrans("+-", "-+"))[::-1]
            for term in inter:
                term[0] = term[0].conjugate() if isinstance(term[0], complex) else term[0]
                term[1:] = term[-1:0:-1]
        return Operator(op_list)

    def __repr__(self):
        return " ".join(f"{J:+}{opstr}{idx}" for opstr, inter in self.op_list for J, *idx in inter)

    # ---- local estimator (operator.py:510-595) --------------------------------------------
    def apply_diag(self, spins_packed: torch.Tensor, n: int) -> torch.Tensor:
        out = torch.empty(spins_packed.shape[0], dtype=torch.float64, device=spins_packed.device)
        c = self.compiled()
        _lib.call("qgx_operator_diag", C.byref(c.struct), _lib.ptr(spins_packed), spins_packed.shape[0], n,
                  _lib.ptr(out), _lib.stream_ptr())
        return out

    def Oloc(self, state, samples) -> torch.Tensor:
        """E_loc(s) = sum_s' <s|O|s'> psi(s')/psi(s) for the samples (device tensor)."""
        from .sampler import Samples
        if not isinstance(samples, Samples):
            samples = Samples.from_spins(samples)
        return state.local_energy(self, samples)

    @staticmethod
    def Oloc_batched(terms) -> list:
        """Oloc of several (operator, state, samples) triples: the RBM states' local energies in
        as few launches as their shapes allow (qgx_rbm_eloc_batched, one per hidden-unit width
        class), each bit for bit its own Oloc; other states are evaluated one by one."""
        from .sampler import Samples
        out = [None] * len(terms)
        jobs, keep = [], []
        for k, (op, state, samples) in enumerate(terms):
            if not isinstance(samples, Samples):
                samples = Samples.from_spins(samples)
            if state.model.kind != "rbm" or state.symm_dev is not None:
                out[k] = state.local_energy(op, samples)
                continue
            comp = op.compiled()
            if comp.max_site >= state.Nmodes:
                raise ValueError("the operator acts on sites beyond the state's lattice")
            e = torch.empty(samples.nsamples, dtype=torch.float64, device=state.params.device)
            out[k] = e
            keep.append(comp)
            jobs.append(_lib.RbmElocJob(_lib.ptr(state.table), state.model.N, state.model.M,
                                        C.pointer(comp.struct), _lib.ptr(samples.packed), samples.nsamples,
                                        _lib.ptr(e)))
        for i in range(0, len(jobs), _lib.RBM_BATCH_MAX_JOBS):
            chunk = jobs[i:i + _lib.RBM_BATCH_MAX_JOBS]
            arr = (_lib.RbmElocJob * len(chunk))(*chunk)
            launches = C.c_int32(0)
            _lib.call("qgx_rbm_eloc_batched", arr, len(chunk), C.byref(launches), _lib.stream_ptr())
        return out

    def expectation(self, state, samples, return_var: bool = False):
        r = samples.reweight_factor
        E = self.Oloc(state, samples)
        w = torch.ones_like(E.real if E.is_complex() else E) if r is None else r
        Em = torch.mean(E * w)
        if return_var:
            var = torch.mean(torch.abs(E) ** 2 * w) - torch.abs(Em) ** 2
            return float(Em.real), float(var.real)
        return float(Em.real)

    # ---- exact diagonalisation (operator.py:331-359), small systems only -------------------
    def to_sparse(self, nup=None, return_states: bool = False):
        """Sparse H in the computational basis (bit i of a state's index = site i up), on the
        sector with nup up spins when given; return_states also returns those basis indices."""
        n = get_sites().N
        if n > 30:
            raise ValueError("exact diagonalisation is limited to N <= 30 sites")
        c0, z, zz, f1, f2 = compile_op_list(self._op_list)
        allb = np.arange(1 << n, dtype=np.int64)
        if nup is not None:
            pc = np.zeros_like(allb)
            for i in range(n):
                pc += (allb >> i) & 1
            states = allb[pc == nup]
        else:
            states = allb
        lookup = np.full(1 << n, -1, dtype=np.int64)
        lookup[states] = np.arange(len(states))
        spin = lambda i: ((states >> i) & 1) * 2 - 1
        diag = np.full(len(states), c0, dtype=np.float64)
        for i, J in z.items():
            diag += J * spin(i)
        for (i, j), J in zz.items():
            diag += J * spin(i) * spin(j)
        rows, cols, vals = [np.arange(len(states))], [np.arange(len(states))], [diag]
        for i, (jm, jp) in f1.items():
            el = np.where(spin(i) > 0, jp, jm)
            ok = el != 0
            rows.append(np.flatnonzero(ok)); cols.append(lookup[states[ok] ^ (1 << i)]); vals.append(el[ok])
        for (i, j), e in f2.items():
            el = np.asarray(e)[2 * (spin(i) > 0) + (spin(j) > 0)]
            tgt = lookup[states ^ ((1 << i) | (1 << j))]
            ok = (el != 0) & (tgt >= 0)
            rows.append(np.flatnonzero(ok)); cols.append(tgt[ok]); vals.append(el[ok])
        m = len(states)
        H = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(m, m))
        return (H, states) if return_states else H

    def todense(self, nup=None) -> np.ndarray:
        return self.to_sparse(nup).toarray()

    def diagonalize(self, symm=None, k: Union[int, str] = 1, nup=None):
        """Lowest k eigenpairs (operator.py:331-359), on the sites' fixed-magnetisation sector
        when Nparticles is given. With a symmetry, the spectrum of H inside the symmetry sector:
        the lowest eigenvalues of P (H - c) P + c, P = sum_g w_g T_g the sector's projector
        (Symmetry.symmetrize), c >= ||H|| so that P's null space lies above every sector
        energy. The reference builds the reduced QuSpin basis instead; here the eigenvectors
        are returned in the full (fixed-magnetisation) computational basis, normalised."""
        sites = get_sites()
        if nup is None and isinstance(sites.Nparticles, tuple):
            nup = sites.Nparticles[0]
        H, states = self.to_sparse(nup, return_states=True)
        if symm is None or symm.is_identity:
            if k == "full" or H.shape[0] <= 256:
                w, v = np.linalg.eigh(H.toarray())
                return (w, v) if k == "full" else (w[:k], v[:, :k])
            return spla.eigsh(H, k=k, which="SA", tol=1e-12)
        P = self._sector_projector(symm, states)
        c = float(abs(H).sum(axis=1).max())  # an upper bound of ||H||_2
        D = H.shape[0]
        if k == "full" or D <= 256:
            w, v = np.linalg.eigh((P @ (H - c * sp.identity(D)) @ P).toarray())
            keep = w < -1e-9 * c
            w, v = w[keep] + c, v[:, keep]
            return (w, v) if k == "full" else (w[:k], v[:, :k])
        Hc = (H - c * sp.identity(D)).tocsr()
        op = spla.LinearOperator((D, D), matvec=lambda x: P @ (Hc @ (P @ x)), dtype=P.dtype)
        v0 = P @ np.random.default_rng(0).normal(size=D).astype(P.dtype)
        w, v = spla.eigsh(op, k=k, which="SA", v0=v0, tol=1e-12)
        order = np.argsort(w)
        v = v[:, order]
        return w[order] + c, v / np.linalg.norm(v, axis=0, keepdims=True)

    @staticmethod
    def _sector_projector(symm, states):
        """(P x)(s) = sum_g w_g x(T_g s) on the basis `states` (sparse, D x D)."""
        n = get_sites().N
        spins = ((states[:, None] >> np.arange(n)) & 1).astype(np.int64)  # 1 = up
        lookup = {int(c): i for i, c in enumerate(states)}
        weights = symm.weights()
        perms = symm.perm
        rows, cols, vals = [], [], []
        D = len(states)
        for g, w in enumerate(weights):
            bits = spins[:, perms[g % len(perms)]]
            if g >= len(perms):
                bits = 1 - bits  # Z2 inversion
            codes = (bits << np.arange(n)).sum(axis=1)
            try:
                idx = np.fromiter((lookup[int(c)] for c in codes), dtype=np.int64, count=D)
            except KeyError:
                raise ValueError("the symmetry does not preserve the basis (spin inversion needs Nup = N/2)")
            rows.append(np.arange(D)); cols.append(idx); vals.append(np.full(D, w))
        dtype = np.complex128 if np.iscomplexobj(weights) and np.any(np.imag(weights) != 0) else np.float64
        vals = np.concatenate(vals).astype(dtype) if dtype == np.complex128 else np.real(np.concatenate(vals))
        return sp.csr_matrix((vals, (np.concatenate(rows), np.concatenate(cols))), shape=(D, D))


# ---- site operators (site_operator.py:8-132) ------------------------------------------------
def _site_op(index, opstr, strength=1.0):
    sites = get_sites()
    if len(index) == 1 and 0 <= index[0] < sites.Nsites:
        idx = int(index[0])
    else:
        shape = sites.shape
        xyz = [0] + [x % l for x, l in zip(index, shape[1:])]
        idx = int(sites.index_from_xyz[tuple(xyz)])
    return Operator([[opstr, [[strength, idx]]]])


def sigma_x(*index) -> Operator:
    return _site_op(index, "x", 2.0)


def sigma_z(*index) -> Operator:
    return _site_op(index, "z", 2.0)


def sigma_p(*index) -> Operator:
    return _site_op(index, "+")


def sigma_m(*index) -> Operator:
    return _site_op(index, "-")


def Ising(h: Number = 0.0, J: Number = 1.0) -> Operator:
    """H = -J sum_<ij> sz_i sz_j - h sum_i sx_i (common_operators.py:56-71)."""
    sites = get_sites()
    H = -h * sum(sigma_x(i) for i in range(sites.Nmodes))
    H += -J * sum(sigma_z(int(i)) @ sigma_z(int(j)) for i, j in sites.get_neighbor())
    return H


def Heisenberg(J: Union[Number, Sequence[Number]] = 1.0, n_neighbor: Union[int, Sequence[int]] = 1,
               msr: bool = False) -> Operator:
    """H = sum_n J_n sum_<ij>_n sigma_i . sigma_j (common_operators.py:23-53)."""
    sites = get_sites()
    J = [J] if isinstance(J, Number) else list(J)
    n_neighbor = [n_neighbor] if isinstance(n_neighbor, Number) else list(n_neighbor)
    if len(J) != len(n_neighbor):
        raise ValueError("'J' and 'n_neighbor' should have the same length.")
    neighbors = sites.get_neighbor(n_neighbor)

    def hij(i, j, sign):
        hx = 2 * sign * (sigma_p(i) @ sigma_m(j) + sigma_m(i) @ sigma_p(j))
        return hx + sigma_z(i) @ sigma_z(j)

    H = 0
    for idx, nb in enumerate(neighbors):
        sign = -1 if msr and n_neighbor[idx] == 1 else 1
        H = H + J[idx] * sum(hij(int(i), int(j), sign) for i, j in nb)
    return H
