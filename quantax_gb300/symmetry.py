"""Symmetry projection of spin states (quantax/symmetry/*.py).

A Symmetry holds the permutations T_g of the group's elements (nperm x N, site i of T_g s
takes s[perm[g, i]]) and their characters chi_g; Z2 inversion doubles the group with the
flipped configurations. A state built with symm=... evaluates

    psi_symm(s) = sum_g w_g psi(T_g s),   w_g = chi_0 chi_g / |G|

(Symmetry.symmetrize, quantax/symmetry/symmetry.py:349-392). The group algebra here is host
numpy: orbits of the generators (symmetry.py:11-57), products of symmetries (:394-432) and
the lattice maps of Translation / LinearTransform (translation.py:7-53,
common_symmetries.py:78-118). The device receives the permutation table (int16) and the
weights w_g (complex, FP64) once, through qgx_symm_t.

Spin systems only: the fermionic permutation signs (symmetry.py:60-86) have no use without
fermionic models, and a generator_sign other than all ones is refused.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence, Tuple, Union

import numpy as np
import torch

from . import _lib
from .global_defs import PARTICLE_TYPE, device, get_lattice, get_sites, is_default_cpl


def _orbit_product(generators: np.ndarray, sectors, complex_chars: bool) -> Tuple[np.ndarray, np.ndarray]:
    """All products g_1^m g_2^n ... of the generators and their characters
    exp(-2 pi i (m q_1 / M + n q_2 / N ...)) (symmetry.py:11-57)."""
    n = generators.shape[1]
    ident = np.arange(n)
    if np.array_equal(generators, np.atleast_2d(ident)) or all(np.array_equal(g, ident) for g in generators):
        return ident[None].copy(), np.ones(1, dtype=np.complex128)
    perm = ident[None].copy()
    chars = np.ones(1, dtype=np.complex128)
    for g, sec in zip(generators, sectors):
        orbit = [ident]
        cur = g.copy()
        while not np.array_equal(cur, ident):
            orbit.append(cur)
            cur = cur[g]
            if len(orbit) > n * n + 1:
                raise ValueError("the generator does not generate a finite cyclic group")
        orbit = np.stack(orbit)
        period = orbit.shape[0]
        if not 0 <= sec < period:
            raise ValueError(f"Sector {sec} out of range.")
        if not complex_chars:
            if (2 * sec) % period != 0:
                raise ValueError("Default dtype is real, but got complex characters.")
            chi = -1.0 if sec else 1.0
        else:
            chi = np.exp(-2j * np.pi * sec / period)
        new_chars = chi ** np.arange(period)
        # element (a, b) applies orbit[b] inside perm[a]: row a of perm indexed by orbit[b]
        perm = perm[:, orbit].reshape(-1, n)
        chars = np.outer(chars, new_chars).reshape(-1)
    return perm, chars


class Symmetry:
    """Symmetry of the system (symmetry.py:89-432), spin systems."""

    def __init__(self, generator: Optional[np.ndarray] = None, sector: Union[int, Sequence] = 0,
                 generator_sign: Optional[np.ndarray] = None, Z2_inversion: int = 0, perm=None, character=None,
                 perm_sign=None):
        sites = get_sites()
        if sites.is_fermion:
            raise NotImplementedError("symmetry projection is built for spin systems")
        self._Nmodes = sites.Nmodes
        self._Nparticles = sites.Nparticles
        n = self._Nmodes
        if generator is None:
            generator = np.arange(n)[None]
        else:
            generator = np.atleast_2d(np.asarray(generator)).astype(np.int64)
            if generator.shape[1] != n:
                raise ValueError(f"Got a generator with size {generator.shape[1]}, incompatible with "
                                 f"the system size {n}.")
        self._generator = generator
        if generator_sign is not None and not np.all(np.asarray(generator_sign) == 1):
            raise NotImplementedError("permutation signs arise only for fermions")
        self._sector = [sector] * generator.shape[0] if isinstance(sector, (int, np.integer)) \
            else np.asarray(sector).reshape(-1).tolist()
        if Z2_inversion not in (-1, 0, 1):
            raise ValueError("Z2_inversion must be -1, 0 or 1")
        self._Z2_inversion = int(Z2_inversion)
        if perm is None or character is None:
            p, c = _orbit_product(generator, self._sector, is_default_cpl())
            perm = p if perm is None else perm
            character = c if character is None else character
        self._perm = np.asarray(perm, dtype=np.int64).reshape(-1, n)
        if not np.array_equal(np.sort(self._perm, axis=1), np.broadcast_to(np.arange(n), self._perm.shape)):
            raise ValueError("every row of perm must be a permutation of the sites")
        self._character = np.asarray(character, dtype=np.complex128).reshape(-1)
        if self._character.size != self._perm.shape[0]:
            raise ValueError("one character per permutation is needed")
        if not is_default_cpl() and np.any(self._character.imag != 0):
            raise ValueError("Default dtype is real, but got complex characters.")
        self._dev = None

    # ---- properties (symmetry.py:188-245) ------------------------------------------------
    @property
    def Nsites(self) -> int:
        return self._Nmodes

    @property
    def Nmodes(self) -> int:
        return self._Nmodes

    @property
    def Nparticles(self):
        return self._Nparticles

    @property
    def particle_type(self):
        return PARTICLE_TYPE.spin

    @property
    def is_fermion(self) -> bool:
        return False

    @property
    def character(self) -> np.ndarray:
        """Characters chi of the permutations (without the Z2 copies)."""
        c = self._character
        return c if is_default_cpl() else c.real

    @property
    def perm(self) -> np.ndarray:
        return self._perm.copy()

    @property
    def nperm(self) -> int:
        return int(self._perm.shape[0])

    @property
    def nsymm(self) -> int:
        """Number of elements in the symmetry group."""
        return self.nperm * (2 if self._Z2_inversion else 1)

    @property
    def Z2_inversion(self) -> int:
        return self._Z2_inversion

    @property
    def is_identity(self) -> bool:
        return self.nsymm == 1

    def weights(self) -> np.ndarray:
        """w_g = chi_0 chi_g / |G| over all nsymm elements, Z2 copies last (symmetry.py:388-391)."""
        c = self._character
        if self._Z2_inversion:
            c = np.concatenate([c, self._Z2_inversion * c])
        return c * c[0] / c.size

    # ---- reference operations ------------------------------------------------------------
    def get_symm_spins(self, spins) -> np.ndarray:
        """All T_g s of one configuration, (nsymm, N) (symmetry.py:325-347)."""
        s = np.asarray(spins)
        if s.ndim > 1:
            raise ValueError(f"Input spins should be 1D, got dimension {s.ndim}")
        out = s[self._perm]
        if self._Z2_inversion:
            out = np.concatenate([out, -out], axis=-2)
        return out

    def symmetrize(self, psi, spins=None):
        """sum_g w_g psi_g of the wavefunctions psi(T_g s) (symmetry.py:349-392)."""
        p = np.asarray(psi.cpu() if isinstance(psi, torch.Tensor) else psi)
        if p.ndim > 1:
            raise ValueError(f"Input wavefunction should be 1D, got dimension {p.ndim}")
        w = self.weights()
        return (p * (w if np.iscomplexobj(p) or is_default_cpl() else w.real)).sum()

    def __matmul__(self, other: "Symmetry") -> "Symmetry":
        """Product group of two symmetries (symmetry.py:394-432)."""
        generator = np.concatenate([self._generator, other._generator], axis=0)
        sector = [*self._sector, *other._sector]
        perm = self._perm[:, other._perm].reshape(-1, self.Nmodes)
        character = np.outer(self._character, other._character).reshape(-1)
        if self._Z2_inversion == 0:
            z2 = other._Z2_inversion
        elif other._Z2_inversion == 0 or self._Z2_inversion == other._Z2_inversion:
            z2 = self._Z2_inversion
        else:
            raise ValueError("Symmetry with different Z2_inversion can't be added")
        return Symmetry(generator, sector, None, z2, perm, character)

    # ---- device form -----------------------------------------------------------------------
    def device_struct(self):
        """The qgx_symm_t of this group on the current device (tables uploaded once)."""
        if self._dev is None:
            if self.nsymm > 1024:
                raise ValueError("the device kernels take at most 1024 group elements")
            perm = torch.as_tensor(self._perm.astype(np.int16), device=device()).contiguous()
            w = self.weights()
            wt = torch.as_tensor(np.stack([w.real, w.imag], axis=1).reshape(-1), dtype=torch.float64,
                                 device=device()).contiguous()
            st = _lib.Symm(C.c_void_p(perm.data_ptr()), C.c_void_p(wt.data_ptr()), self.nperm, self._Z2_inversion)
            self._dev = (perm, wt, st)
        return self._dev[2]


# ---- common symmetries (common_symmetries.py, translation.py) -----------------------------
_identity = None
_z2 = {}


def Identity() -> Symmetry:
    """Identity (no symmetry)."""
    global _identity
    if _identity is None or _identity.Nmodes != get_sites().Nmodes:
        _identity = Symmetry()
    return _identity


def Z2Inversion(eigval: int = 1) -> Symmetry:
    """Spin flip s -> -s with eigenvalue eigval (common_symmetries.py:21-40)."""
    if eigval not in (1, -1):
        raise ValueError("'eigval' of Z2Inversion should be 1 or -1.")
    key = (eigval, get_sites().Nmodes)
    if key not in _z2:
        _z2[key] = Symmetry(Z2_inversion=eigval)
    return _z2[key]


def SpinInverse(eigval: int = 1) -> Symmetry:
    """Flips all spins (common_symmetries.py:43-71): Z2Inversion in spin systems."""
    return Z2Inversion(eigval)


def ParticleHole(eigval: int = 1) -> Symmetry:
    raise RuntimeError("`ParticleHole` symmetry is only for fermion systems.")


def _standardize_coord(coord: np.ndarray) -> np.ndarray:
    """Fold coordinates into the periodic cell (common_symmetries.py:92-104)."""
    lat = get_lattice()
    basis = lat.basis_vectors.T
    xyz = np.linalg.solve(basis, coord.T).T
    periodic = lat.boundary != 0
    ext = np.asarray(lat.shape, dtype=float)[1:][periodic]
    sh = xyz[:, periodic] % ext
    sh[np.isclose(sh, ext)] = 0.0
    xyz[:, periodic] = sh
    return xyz @ lat.basis_vectors


def LinearTransform(matrix: np.ndarray, center: Optional[np.ndarray] = None, sector: int = 0,
                    character=None) -> Symmetry:
    """The permutation a linear map of the lattice induces (common_symmetries.py:107-148)."""
    lat = get_lattice()
    coord = lat.coord
    if center is None:
        center = coord.mean(axis=0)
    base = _standardize_coord(coord)
    moved = _standardize_coord((coord - center) @ np.asarray(matrix, dtype=float).T + center)
    match = np.all(np.isclose(base[:, None, :], moved[None, :, :]), axis=-1)
    if not np.all(match.sum(axis=1) == 1):
        raise ValueError("The transformation does not map the lattice to itself.")
    generator = np.argmax(match, axis=1)
    return Symmetry(generator, sector, character=character)


def Flip(axis: Union[int, Sequence] = 0, center: Optional[np.ndarray] = None, sector: int = 0) -> Symmetry:
    """Mirror along the given axes (common_symmetries.py:151-165)."""
    m = np.ones(get_lattice().ndim)
    m[np.asarray(axis)] = -1
    return LinearTransform(np.diag(m), center, sector)


def Rotation(angle: float, axes: Sequence = (0, 1), center: Optional[np.ndarray] = None, sector: int = 0,
             character=None) -> Symmetry:
    """Rotation by angle in the plane of two axes (common_symmetries.py:168-206)."""
    ndim = get_lattice().ndim
    if max(axes) >= ndim:
        raise ValueError(f"The rotated axis {max(axes)} is out-of-bound for a {ndim}-D system")
    m = np.eye(ndim)
    x, y = axes
    c, s = np.cos(angle), np.sin(angle)
    m[x, x], m[x, y], m[y, x], m[y, y] = c, -s, s, c
    if character is not None:
        character = np.asarray(character, dtype=np.complex128)
    return LinearTransform(m, center, sector, character)


def C4v(center: Optional[np.ndarray] = None, repr: str = "A1") -> Symmetry:
    """C4v point group in one of its irreducible representations (common_symmetries.py:209-241)."""
    sectors = {"A1": (0, 0), "A2": (0, 1), "B1": (2, 0), "B2": (2, 1)}
    if repr in sectors:
        r, f = sectors[repr]
        return Rotation(np.pi / 2, center=center, sector=r) @ Flip(center=center, sector=f)
    if repr == "E":
        return Rotation(np.pi, center=center, character=np.array([2.0, -2.0]))
    raise ValueError("'repr' should be one of the following: 'A1', 'A2', 'B1', 'B2' or 'E'")


def D6(center: Optional[np.ndarray] = None, repr: str = "A1") -> Symmetry:
    """D6 point group (common_symmetries.py:244-278)."""
    sectors = {"A1": (0, 0), "A2": (0, 1), "B1": (3, 0), "B2": (3, 1)}
    if repr in sectors:
        r, f = sectors[repr]
        return Rotation(np.pi / 3, center=center, sector=r) @ Flip(center=center, sector=f)
    chars = {"E1": [2, 1, -1, -2, -1, 1], "E2": [2, -1, -1, 2, -1, -1]}
    if repr in chars:
        return Rotation(np.pi / 3, character=np.asarray(chars[repr], dtype=float))
    raise ValueError("'repr' should be one of the following: 'A1', 'A2', 'B1', 'B2', 'E1' or 'E2'")


class Translation(Symmetry):
    """Translations by the given lattice vectors (translation.py:7-53)."""

    def __init__(self, vectors: Sequence, sector: int = 0):
        lat = get_lattice()
        vectors = np.asarray(vectors, dtype=np.int64).reshape(-1, lat.ndim)
        if np.any((vectors != 0) & (lat.boundary[None, :] == 0)):
            raise ValueError("Translation symmetry can't be imposed on open boundary.")
        shape = np.asarray(lat.shape[1:])
        gens = []
        for vec in vectors:
            for ax, v in enumerate(vec):
                if v != 0 and shape[ax] % v != 0:
                    raise ValueError("Translation vector must be compatible with lattice shape, "
                                     f"got lattice shape {tuple(shape)} and vector {vec}.")
            xyz = lat.xyz_from_index.copy()
            xyz[:, 1:] = (xyz[:, 1:] + vec[None, :]) % shape
            gens.append(lat.index_from_xyz[tuple(xyz.T)])
        self._vectors = vectors
        super().__init__(np.stack(gens), sector)

    @property
    def vectors(self) -> np.ndarray:
        return self._vectors.copy()


def TransND(sector: Union[int, Tuple[int, ...]] = 0) -> Translation:
    """Unit translations along every lattice axis (translation.py:82-87)."""
    return Translation(np.identity(get_lattice().ndim), sector)
