"""Lattices (host-side setup): site indexing, periodic distances and n-th-neighbour bonds.

Mirrors quantax/sites/sites.py:8-283 and quantax/sites/lattice.py:7-179 for hypercubic
grids (Grid, Chain, Square, Cube): site index in C order over the extents, shortest
periodic-image distance, n-th-neighbour pairs (i < j) at the n-th smallest distance in
row-major order.
"""
from __future__ import annotations

from typing import Sequence, Tuple, Union

import numpy as np

from . import global_defs
from .global_defs import PARTICLE_TYPE


class Sites:
    def __init__(self, Nsites: int, particle_type=PARTICLE_TYPE.spin, Nparticles=None, double_occ=None,
                 coord=None):
        if isinstance(particle_type, str):
            particle_type = PARTICLE_TYPE[particle_type.lower().replace(" ", "_")]
        if particle_type != PARTICLE_TYPE.spin:
            raise NotImplementedError("quantax_gb300 implements spin systems only")
        self._Nsites = int(Nsites)
        self._particle_type = particle_type
        if Nparticles is None:
            Nparticles = self._Nsites
        elif isinstance(Nparticles, int):
            if Nparticles != self._Nsites:
                raise ValueError("Specify spin conservation with a tuple (Nup, Ndown).")
        else:
            Nparticles = tuple(int(x) for x in Nparticles)
            if sum(Nparticles) != self._Nsites:
                raise ValueError("The total number of spin-up and spin-down particles should be "
                                 "equal to the number of sites in spin systems.")
        self._Nparticles = Nparticles
        self._double_occ = False if double_occ is None else double_occ
        self._coord = None if coord is None else np.asarray(coord, dtype=float)
        self._neighbors = []
        self._dist = None
        global_defs._set_sites(self)

    @property
    def Nsites(self) -> int:
        return self._Nsites

    @property
    def Nmodes(self) -> int:
        return self._Nsites

    @property
    def N(self) -> int:
        return self._Nsites

    @property
    def particle_type(self):
        return self._particle_type

    @property
    def Nparticles(self):
        return self._Nparticles

    @property
    def is_fermion(self) -> bool:
        return False

    @property
    def double_occ(self) -> bool:
        return self._double_occ

    @property
    def coord(self):
        return self._coord

    @property
    def dist(self) -> np.ndarray:
        if self._dist is None:
            self._dist = self._get_dist()
        return self._dist

    def _get_dist(self) -> np.ndarray:
        c = self._coord
        return np.linalg.norm(c[None, :, :] - c[:, None, :], axis=2)

    def get_neighbor(self, n_neighbor: Union[int, Sequence[int]] = 1):
        max_n = n_neighbor if isinstance(n_neighbor, int) else max(n_neighbor)
        if len(self._neighbors) < max_n:
            self._compute_neighbor(max_n)
        if isinstance(n_neighbor, int):
            return self._neighbors[n_neighbor - 1]
        return [self._neighbors[n - 1] for n in n_neighbor]

    def _compute_neighbor(self, max_neighbor: int) -> None:
        tol = 1e-6
        dist = self.dist
        self._neighbors = []
        min_dist = tol
        for _ in range(max_neighbor):
            min_dist = np.min(dist[dist > min_dist])
            nb = np.argwhere(np.abs((dist - min_dist) / min_dist) < tol)
            nb = nb[nb[:, 0] < nb[:, 1]]
            self._neighbors.append(nb)
            min_dist *= 1 + tol

    def neighbor_table(self, n_neighbor: Union[int, Sequence[int]] = 1) -> np.ndarray:
        """(N, z) int32 neighbour rows padded with -1 (common_samplers.py:36-55)."""
        orders = [n_neighbor] if isinstance(n_neighbor, int) else list(n_neighbor)
        mat = np.zeros((self.N, self.N), dtype=bool)
        for nb in self.get_neighbor(orders):
            mat[nb[:, 0], nb[:, 1]] = True
        mat = mat | mat.T
        z = int(mat.sum(axis=1).max())
        table = np.full((self.N, z), -1, dtype=np.int32)
        for i in range(self.N):
            nz = np.flatnonzero(mat[i])
            table[i, :len(nz)] = nz
        return table


class Lattice(Sites):
    def __init__(self, extent: Sequence[int], basis_vectors, site_offsets=None,
                 boundary: Union[int, Sequence[int]] = 1, particle_type=PARTICLE_TYPE.spin,
                 Nparticles=None, double_occ=None):
        ndim = len(extent)
        self._basis_vectors = np.asarray(basis_vectors, dtype=float)
        self._site_offsets = np.zeros([1, ndim]) if site_offsets is None else np.asarray(site_offsets, float)
        if self._site_offsets.shape[0] != 1:
            raise NotImplementedError("only one site per unit cell is implemented")
        self._shape = (1,) + tuple(int(e) for e in extent)
        self._boundary = np.full(ndim, boundary, dtype=int) if isinstance(boundary, int) \
            else np.asarray(boundary, dtype=int)
        if np.any(self._boundary == -1):
            raise ValueError("Spin system can't have anti-periodic boundary conditions.")
        n = int(np.prod(self._shape))
        idx = np.arange(n)
        xyz = []
        for i in range(len(self._shape)):
            later = int(np.prod(self._shape[i + 1:], dtype=np.int64))
            xyz.append(idx // later % self._shape[i])
        self._xyz_from_index = np.stack(xyz, axis=1)
        self._index_from_xyz = idx.reshape(self._shape)
        coord = self._xyz_from_index[:, 1:].astype(float) @ self._basis_vectors
        super().__init__(n, particle_type, Nparticles, double_occ, coord)

    @property
    def shape(self) -> Tuple[int, ...]:
        return self._shape

    @property
    def ndim(self) -> int:
        return len(self._shape) - 1

    @property
    def basis_vectors(self) -> np.ndarray:
        return self._basis_vectors

    @property
    def ncells(self) -> int:
        return int(np.prod(self._shape[1:]))

    @property
    def boundary(self) -> np.ndarray:
        return self._boundary

    @property
    def index_from_xyz(self):
        return self._index_from_xyz

    @property
    def xyz_from_index(self):
        return self._xyz_from_index

    def _get_dist(self) -> np.ndarray:
        x = self._xyz_from_index[:, 1:].astype(float)
        d = np.abs(x[None, :, :] - x[:, None, :])
        ext = np.asarray(self._shape[1:], dtype=float)
        pbc = self._boundary != 0
        d = np.where(pbc[None, None, :], np.minimum(d, ext - d), d)
        d = d @ np.abs(self._basis_vectors)  # orthogonal grids only
        return np.linalg.norm(d, axis=-1)


class Grid(Lattice):
    def __init__(self, extent, boundary=1, particle_type=PARTICLE_TYPE.spin, Nparticles=None, double_occ=None):
        super().__init__(extent, np.eye(len(extent)), None, boundary, particle_type, Nparticles, double_occ)


def Chain(L: int, boundary=1, particle_type=PARTICLE_TYPE.spin, Nparticles=None, double_occ=None):
    """1D chain lattice."""
    return Grid([L], boundary, particle_type, Nparticles, double_occ)


def Square(L: int, boundary=1, particle_type=PARTICLE_TYPE.spin, Nparticles=None, double_occ=None):
    """2D square lattice."""
    return Grid([L, L], boundary, particle_type, Nparticles, double_occ)


def Cube(L: int, boundary=1, particle_type=PARTICLE_TYPE.spin, Nparticles=None, double_occ=None):
    """3D cube lattice."""
    return Grid([L, L, L], boundary, particle_type, Nparticles, double_occ)
