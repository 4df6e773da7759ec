"""Lattice geometry for the oracle (test infrastructure only).

Restates the reference's n-th-neighbour bond construction for hypercubic grids with
periodic or open boundaries:
  * site index is C-order over the extents (quantax/sites/lattice.py:69-76);
  * the distance between two sites is the shortest periodic image distance
    (quantax/sites/lattice.py:139-179);
  * the n-th-neighbour bonds are the pairs (i, j), i < j, whose distance equals the
    n-th smallest non-zero distance, listed in row-major (argwhere) order
    (quantax/sites/sites.py:267-283).

Pinned: coordinates and bonds equal the output of the reference's own sites code for the
lattices in tests/golden/lattice_reference.json.
"""
from __future__ import annotations

import numpy as np


def coords(extent):
    extent = tuple(int(e) for e in extent)
    n = int(np.prod(extent))
    idx = np.arange(n)
    xyz = []
    for i in range(len(extent)):
        later = int(np.prod(extent[i + 1:], dtype=np.int64))
        xyz.append(idx // later % extent[i])
    return np.stack(xyz, axis=1)


def distances(extent, pbc=True):
    xyz = coords(extent).astype(np.float64)
    d = xyz[:, None, :] - xyz[None, :, :]
    if pbc:
        ext = np.asarray(extent, dtype=np.float64)
        d = np.abs(d)
        d = np.minimum(d, ext - d)
    return np.linalg.norm(d, axis=-1)


def neighbors(extent, n_neighbor=1, pbc=True):
    """List of (nb, 2) int arrays, one per requested neighbour order."""
    single = isinstance(n_neighbor, int)
    orders = [n_neighbor] if single else list(n_neighbor)
    dist = distances(extent, pbc)
    tol = 1e-6
    out = []
    min_dist = tol
    shells = []
    for _ in range(max(orders)):
        min_dist = np.min(dist[dist > min_dist])
        nb = np.argwhere(np.abs((dist - min_dist) / min_dist) < tol)
        nb = nb[nb[:, 0] < nb[:, 1]]
        shells.append(nb)
        min_dist *= 1 + tol
    for o in orders:
        out.append(shells[o - 1])
    return out[0] if single else out


def neighbor_table(extent, n_neighbor=1, pbc=True):
    """Per-site neighbour rows padded with -1 (quantax/sampler/common_samplers.py:36-55)."""
    orders = [n_neighbor] if isinstance(n_neighbor, int) else list(n_neighbor)
    n = int(np.prod(extent))
    mat = np.zeros((n, n), dtype=bool)
    for nb in neighbors(extent, orders, pbc):
        mat[nb[:, 0], nb[:, 1]] = True
    mat = mat | mat.T
    z = int(mat.sum(axis=1).max())
    table = np.full((n, z), -1, dtype=np.int32)
    for i in range(n):
        nz = np.flatnonzero(mat[i])
        table[i, :len(nz)] = nz
    return table
