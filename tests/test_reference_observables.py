"""Operator conventions and algebra pinned to values the reference's notebooks print.

tutorials/samples.ipynb (Square(4), no particle-number constraint): <M2> of the Ising(h=3)
and Ising(h=1) ground states with M = sum_i sigma_z(i) / N, M2 = M @ M (:142, :342, :411), and
the squared overlap of the two ground states (:451). tutorials/exact_diag.ipynb (4x4
Heisenberg(), Sz = 0 sector): the spin correlations <C01>, <C02> (:227-228) and the ground
state's amplitude at a printed configuration (:160-161). Both the oracle (op lists built by
hand in the reference's QuSpin format) and the package (its Operator algebra: sigma_z,
sigma_p, sigma_m, sums, products, Ising, Heisenberg, diagonalize) must reproduce them.
"""
import json
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from oracle import lattice, operators as ops

GOLDEN = json.loads((Path(__file__).parent / "golden" / "reference_energies.json").read_text())
N = 16


def _lowest(H):
    # k = 2: the Ising(h=1) ground state lies 5.5e-7 below the next level on this lattice
    w, v = spla.eigsh(H, k=2, which="SA", tol=1e-13)
    return v[:, int(np.argmin(w))]


# ---- oracle ---------------------------------------------------------------------------------
def _oracle_ising_gs(h):
    H, _ = ops.sparse_matrix(N, ops.ising_op_list(N, lattice.neighbors((4, 4), 1), h, 1.0))
    return _lowest(H)


def _oracle_m2():
    # sigma_z(i) is "z" with strength 2 (quantax/operator/site_operator.py:39-132); M @ M
    # concatenates the op strings and multiplies the strengths (operator.py:470-505)
    return ops.sparse_matrix(N, [["zz", [[4.0 / N ** 2, i, j] for i in range(N) for j in range(N)]]])[0]


def _oracle_corr(i, j, nup):
    op_list = [["zz", [[1.0, i, j]]], ["+-", [[0.5, i, j]]], ["-+", [[0.5, i, j]]]]
    return ops.sparse_matrix(N, op_list, nup)


def _oracle_heisenberg_gs():
    H, states = ops.sparse_matrix(N, ops.heisenberg_op_list([lattice.neighbors((4, 4), 1)]), nup=8)
    return _lowest(H), states


@pytest.mark.parametrize("name,h", [("square4_ising_h1_M2", 1.0), ("square4_ising_h3_M2", 3.0)])
def test_oracle_ising_magnetisation(name, h):
    g = GOLDEN[name]
    v = _oracle_ising_gs(h)
    assert abs(v @ (_oracle_m2() @ v) - g["value"]) < 1e-12, g["source"]


def test_oracle_ising_overlap():
    g = GOLDEN["square4_ising_overlap_h1_h3"]
    assert abs((_oracle_ising_gs(1.0) @ _oracle_ising_gs(3.0)) ** 2 - g["value"]) < 1e-12, g["source"]


@pytest.mark.parametrize("name", ["square4_heisenberg_C01", "square4_heisenberg_C02"])
def test_oracle_heisenberg_correlations(name):
    g = GOLDEN[name]
    v, _ = _oracle_heisenberg_gs()
    C, _ = _oracle_corr(g["i"], g["j"], 8)
    assert abs(v @ (C @ v) - g["value"]) < 1e-12, g["source"]


def test_oracle_heisenberg_amplitude():
    g = GOLDEN["square4_heisenberg_psi0_at_s"]
    v, states = _oracle_heisenberg_gs()
    code = sum(1 << i for i, x in enumerate(g["s"]) if x > 0)
    amp = v[int(np.flatnonzero(states == code)[0])]
    assert abs(abs(amp) - g["value"]) < 5e-9, g["source"]  # printed with 6 significant digits


# ---- package ----------------------------------------------------------------------------------
@pytest.fixture
def qtx():
    import quantax_gb300 as q
    yield q
    q.sites.Square(4)  # leave a neutral lattice behind


def _package_m2(qtx):
    from quantax_gb300.operator import sigma_z
    M = sum(sigma_z(i) for i in range(N)) / N
    return (M @ M).to_sparse()


def _package_ising_gs(qtx, h):
    return _lowest(qtx.operator.Ising(h=h).to_sparse())


@pytest.mark.parametrize("name,h", [("square4_ising_h1_M2", 1.0), ("square4_ising_h3_M2", 3.0)])
def test_package_ising_magnetisation(qtx, name, h):
    g = GOLDEN[name]
    qtx.sites.Square(4)
    v = _package_ising_gs(qtx, h)
    assert abs(v @ (_package_m2(qtx) @ v) - g["value"]) < 1e-12, g["source"]


def test_package_ising_overlap(qtx):
    g = GOLDEN["square4_ising_overlap_h1_h3"]
    qtx.sites.Square(4)
    assert abs((_package_ising_gs(qtx, 1.0) @ _package_ising_gs(qtx, 3.0)) ** 2 - g["value"]) < 1e-12


def _package_corr(i, j):
    from quantax_gb300.operator import sigma_m, sigma_p, sigma_z
    return (sigma_z(i) @ sigma_z(j) + 2 * sigma_p(i) @ sigma_m(j) + 2 * sigma_m(i) @ sigma_p(j)) / 4


def test_package_heisenberg_correlations_and_amplitude(qtx):
    qtx.sites.Square(4, Nparticles=(8, 8))
    H = qtx.operator.Heisenberg()
    w, v = H.diagonalize(k=2)
    v0 = v[:, 0]
    _, states = H.to_sparse(8, return_states=True)
    assert abs(w[0] - GOLDEN["square4_heisenberg_E0"]["value"]) < 1e-10
    for name in ("square4_heisenberg_C01", "square4_heisenberg_C02"):
        g = GOLDEN[name]
        C = _package_corr(g["i"], g["j"]).to_sparse(8)
        assert abs(v0 @ (C @ v0) - g["value"]) < 1e-12, g["source"]
    g = GOLDEN["square4_heisenberg_psi0_at_s"]
    code = sum(1 << i for i, x in enumerate(g["s"]) if x > 0)
    assert abs(abs(v0[int(np.flatnonzero(states == code)[0])]) - g["value"]) < 5e-9, g["source"]
