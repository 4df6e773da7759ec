"""Symmetry projection on the host: the oracle pinned against the reference's exact energies,
and the package's group construction (quantax_gb300.symmetry) against the oracle."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import lattice, operators, symmetry as osym

GOLDEN = Path(__file__).parent / "golden"


def _full_group(L, complex_chars=True):
    """TransND() @ Rotation(pi/2) @ Flip() @ SpinInverse(): the full_symm of the J1-J2 notebook."""
    g = osym.group([osym.translation(L, 1, 0), osym.translation(L, 0, 1)], [0, 0], complex_chars)
    g = osym.product(g, osym.group([osym.rotation90(L)], [0], complex_chars))
    return osym.product(g, osym.group([osym.flip0(L)], [0], complex_chars))


@pytest.mark.parametrize("name", ["square4_heisenberg_msr_E0", "square4_j1j2_0.5_msr_E0"])
def test_sector_ed_matches_reference_notebooks(name):
    """ED inside the fully symmetric sector of TransND @ Rotation(pi/2) @ Flip @ SpinInverse
    gives the ground energy the reference's H.diagonalize(full_symm) printed."""
    g = json.loads((GOLDEN / "reference_energies.json").read_text())[name]
    shells = lattice.neighbors((4, 4), g["n_neighbor"])
    H, states = operators.sparse_matrix(16, operators.heisenberg_op_list(shells, g["J"], g["n_neighbor"], g["msr"]),
                                        nup=8)
    basis = ((states[:, None] >> np.arange(16)) & 1) * 2 - 1
    perms, chars = _full_group(4)
    assert perms.shape[0] == 128 and len({tuple(p) for p in perms}) == 128
    e = osym.sector_ground_energy(H, basis, perms, chars, z2=1)
    assert abs(e[0] - g["value"]) < 1e-9


def test_z2_odd_sector_is_the_triplet():
    """The lowest state odd under spin inversion is the first excited state the reference's
    exact-diagonalisation notebook printed (the S = 1 triplet)."""
    g = json.loads((GOLDEN / "reference_energies.json").read_text())["square4_heisenberg_E1"]
    shells = lattice.neighbors((4, 4), [1])
    H, states = operators.sparse_matrix(16, operators.heisenberg_op_list(shells, [1.0], [1], False), nup=8)
    basis = ((states[:, None] >> np.arange(16)) & 1) * 2 - 1
    e = osym.sector_ground_energy(H, basis, np.arange(16)[None], np.ones(1), z2=-1)
    assert abs(e[0] - g["value"]) < 1e-9


def test_projection_transforms_with_the_character():
    """For a one-dimensional representation psi_symm(T_h s) = psi_symm(s) / chi_h (abelian
    translations, complex sectors) and psi_symm(-s) = z2 psi_symm(s)."""
    L = 4
    perms, chars = osym.group([osym.translation(L, 1, 0), osym.translation(L, 0, 1)], [1, 3])
    rng = np.random.default_rng(0)
    A = rng.normal(size=(16, 16)) + 1j * rng.normal(size=(16, 16))
    a = rng.normal(size=16)  # an odd part, so that the Z2-odd projection does not vanish
    log_psi = lambda x: 0.3 * (x @ a) + np.log(np.cosh(x @ A * 0.2)).sum(axis=-1)
    s = rng.choice([-1, 1], size=(5, 16))
    base = osym.log_psi_symm(log_psi, s, perms, chars, z2=-1)
    for h in (1, 5, 11):
        moved = osym.log_psi_symm(log_psi, s[:, perms[h]], perms, chars, z2=-1)
        # configurations whose projection vanishes by symmetry give 0 up to rounding
        np.testing.assert_allclose(np.exp(moved) * chars[h], np.exp(base), rtol=1e-10, atol=1e-12)
    flipped = osym.log_psi_symm(log_psi, -s, perms, chars, z2=-1)
    np.testing.assert_allclose(np.exp(flipped), -np.exp(base), rtol=1e-10, atol=1e-12)
    assert np.abs(np.exp(base)).max() > 1.0


def _pairs(perms, chars):
    return sorted((tuple(int(v) for v in p), complex(np.round(c, 12))) for p, c in zip(perms, chars))


@pytest.mark.parametrize("case", ["C4v-A1", "C4v-B2", "C4v-E", "trans-sector", "full"])
def test_package_group_matches_oracle(case):
    import quantax_gb300 as qtx
    from quantax_gb300 import symmetry as S
    qtx.set_default_dtype(np.complex128)
    try:
        qtx.sites.Square(4, Nparticles=(8, 8))
        L = 4
        if case.startswith("C4v"):
            rep = case.split("-")[1]
            sym = S.C4v(repr=rep)
            if rep == "E":
                pr = osym.group([osym.rotation90(L)[osym.rotation90(L)]], [0])
                want = (pr[0], np.array([2.0, -2.0]))
            else:
                r, f = {"A1": (0, 0), "B2": (2, 1)}[rep]
                want = osym.product(osym.group([osym.rotation90(L)], [r]), osym.group([osym.flip0(L)], [f]))
        elif case == "trans-sector":
            sym = S.TransND(sector=(1, 2))
            want = osym.group([osym.translation(L, 1, 0), osym.translation(L, 0, 1)], [1, 2])
        else:
            sym = S.TransND() @ S.Rotation(np.pi / 2) @ S.Flip() @ S.SpinInverse()
            want = _full_group(L)
            assert sym.Z2_inversion == 1 and sym.nsymm == 256
        assert _pairs(sym.perm, sym._character) == _pairs(*want)
        # the identity comes first, so the weights chi_0 chi_g / |G| agree element by element
        assert np.array_equal(sym.perm[0], np.arange(16)) and np.array_equal(want[0][0], np.arange(16))
        w = sym.weights()[:sym.nperm]
        w_want = osym.weights(want[1], sym.Z2_inversion)[:sym.nperm]
        assert _pairs(sym.perm, w) == _pairs(want[0], w_want)
    finally:
        qtx.set_default_dtype(np.float64)


def test_package_real_dtype_rules():
    """Complex characters with a real default dtype are refused (symmetry.py:41-45); sector 2
    of a period-4 rotation is the real character -1."""
    import quantax_gb300 as qtx
    from quantax_gb300 import symmetry as S
    qtx.set_default_dtype(np.float64)
    qtx.sites.Square(4, Nparticles=(8, 8))
    with pytest.raises(ValueError, match="complex characters"):
        S.Rotation(np.pi / 2, sector=1)
    r = S.Rotation(np.pi / 2, sector=2)
    np.testing.assert_array_equal(r.character, [1, -1, 1, -1])
    with pytest.raises(ValueError):
        S.Z2Inversion(0)
    assert (S.SpinInverse(-1)).weights().tolist() == [0.5, -0.5]


@pytest.mark.parametrize("name", ["square4_heisenberg_msr_E0", "square4_j1j2_0.5_msr_E0"])
def test_package_diagonalize_with_symmetry(name):
    """Operator.diagonalize(full_symm) as the J1-J2 notebook calls it (cells 5, 21) gives the
    energy the reference printed; the Z2-odd sector gives the triplet of exact_diag.ipynb."""
    import quantax_gb300 as qtx
    from quantax_gb300.symmetry import Flip, Rotation, SpinInverse, TransND
    g = json.loads((GOLDEN / "reference_energies.json").read_text())[name]
    qtx.set_default_dtype(np.float64)
    qtx.sites.Square(4, Nparticles=(8, 8))
    H = qtx.operator.Heisenberg(J=g["J"], n_neighbor=g["n_neighbor"], msr=g["msr"])
    full_symm = TransND() @ Rotation(np.pi / 2) @ Flip() @ SpinInverse()
    E, wf = H.diagonalize(full_symm)
    assert abs(E[0] - g["value"]) < 1e-9
    # the eigenvector is symmetric: projecting it again changes nothing
    assert wf.shape[0] == 12870 and abs(np.linalg.norm(wf[:, 0]) - 1) < 1e-9


def test_package_diagonalize_z2_odd_sector():
    import quantax_gb300 as qtx
    from quantax_gb300.symmetry import SpinInverse
    g = json.loads((GOLDEN / "reference_energies.json").read_text())["square4_heisenberg_E1"]
    qtx.set_default_dtype(np.float64)
    qtx.sites.Square(4, Nparticles=(8, 8))
    H = qtx.operator.Heisenberg(J=[1.0], n_neighbor=[1], msr=False)
    E, _ = H.diagonalize(SpinInverse(-1))
    assert abs(E[0] - g["value"]) < 1e-9
