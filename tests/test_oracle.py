"""The CPU oracle against the reference's known answers and its own consistency."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import lattice, metropolis, operators, philox, rbm, sr

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_philox_known_answers():
    # published Random123 known-answer vectors for philox4x32-10
    cases = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, want in cases:
        assert philox.philox4x32_10(ctr, key).tolist() == want


@pytest.mark.parametrize("name", ["square4_heisenberg_msr_E0", "square4_j1j2_0.5_msr_E0", "square4_heisenberg_E0"])
def test_ed_matches_reference_notebooks(name):
    g = json.loads((GOLDEN / "reference_energies.json").read_text())[name]
    shells = lattice.neighbors((g["L"], g["L"]), g["n_neighbor"])
    ops = operators.heisenberg_op_list(shells, g["J"], g["n_neighbor"], g["msr"])
    e0 = operators.ground_energy(g["L"] ** 2, ops, nup=g["nup"])
    assert abs(e0 - g["value"]) < 1e-10


def test_ed_excited_state_matches_reference():
    g = json.loads((GOLDEN / "reference_energies.json").read_text())["square4_heisenberg_E1"]
    shells = lattice.neighbors((4, 4), [1])
    H, _ = operators.sparse_matrix(16, operators.heisenberg_op_list(shells, [1.0], [1], False), nup=8)
    import scipy.sparse.linalg as spla
    w = np.sort(spla.eigsh(H, k=2, which="SA", tol=1e-12)[0])
    assert abs(w[1] - g["value"]) < 1e-9


def test_tfim_chain8_ground_energy():
    assert abs(operators.ground_energy(8, operators.chain_tfim(8)) - (-10.2516617909660)) < 1e-10


def test_neighbours():
    assert lattice.neighbors((8,), 1).shape == (8, 2)
    nn, nnn = lattice.neighbors((10, 10), [1, 2])
    assert nn.shape == (200, 2) and nnn.shape == (200, 2)
    t = lattice.neighbor_table((10, 10), 1)
    assert t.shape == (100, 4) and (t >= 0).all()


def test_rbm_local_update_matches_direct():
    # mirrors tutorials/local_updates.ipynb: local-update psi == direct psi
    W, b, a = rbm.init_normal(16, 32, 0.2, seed=1, visible_bias=True)
    net = rbm.RBM(W, b, a)
    s = metropolis.init_uniform(5, 16, 3)
    th = net.theta(s)
    k = 7
    s2 = s.copy()
    s2[:, k] *= -1
    th2 = th + 2 * np.outer(s2[:, k], net.W[:, k])
    direct = net.log_psi(s2)
    local = rbm.logcosh(th2).sum(axis=1) + s2 @ net.a
    np.testing.assert_allclose(local, direct, rtol=1e-12)


def test_rbm_jacobian_finite_difference():
    W, b, a = rbm.init_normal(6, 5, 0.3, seed=2, visible_bias=True)
    net = rbm.RBM(W, b, a)
    s = metropolis.init_uniform(3, 6, 4)
    O = net.jacobian(s)
    p0 = net.params()
    eps = 1e-6
    for k in [0, 7, 29, 31, 36]:
        p = p0.copy(); p[k] += eps
        net.set_params(p); lp1 = net.log_psi(s)
        p = p0.copy(); p[k] -= eps
        net.set_params(p); lp0 = net.log_psi(s)
        np.testing.assert_allclose((lp1 - lp0) / (2 * eps), O[:, k], rtol=1e-6, atol=1e-9)
    net.set_params(p0)


def test_init_fixed_up_is_permutation():
    s = metropolis.init_fixed_up(50, 100, 50, 7)
    assert (np.sum(s > 0, axis=1) == 50).all()
    assert len({tuple(r) for r in s}) == 50


def test_sampler_detailed_balance_small():
    # exact |psi|^2 of a 4-site RBM vs the LocalFlip histogram
    W, b, a = rbm.init_normal(4, 3, 0.4, seed=5, visible_bias=True)
    net = rbm.RBM(W, b, a)
    states = np.array([[1 if (x >> i) & 1 else -1 for i in range(4)] for x in range(16)])
    p = np.exp(2 * net.log_psi(states)); p /= p.sum()
    s = metropolis.init_uniform(4000, 4, 1)
    s, _, _ = metropolis.sweep(net.log_psi, s, 200, seed=2)
    idx = ((s > 0).astype(int) << np.arange(4)).sum(axis=1)
    hist = np.bincount(idx, minlength=16) / len(idx)
    assert np.abs(hist - p).max() < 0.02


def test_sr_branches_agree():
    rng = np.random.default_rng(0)
    A = rng.normal(size=(20, 50)); b = rng.normal(size=20)
    x1 = sr.minnorm_shift(A, b, ashift=1e-3)
    # min-norm shift solution == A^T (AA^T + eps)^-1 b == (A^T A + eps)^-1 A^T b
    x2 = sr.lstsq_shift(A, b, ashift=1e-3)
    tr = np.trace(A @ A.T)
    # the relative parts of the shifts differ (trace of T vs S are equal), so they agree
    np.testing.assert_allclose(x1, x2, rtol=1e-8, atol=1e-10)
    x3 = sr.minnorm_pinv(A, b, rtol=1e-12)
    np.testing.assert_allclose(A @ x3, b, rtol=1e-8, atol=1e-8)
    assert tr > 0


def test_golden_oracle_fixture_stable():
    g = json.loads((GOLDEN / "oracle_small.json").read_text())
    ctr = philox.stream_counter(np.arange(4), np.arange(4), philox.TAG_PROPOSE)
    assert philox.philox4x32_10(ctr, philox.seed_key(123)).tolist() == g["philox_seed123"]
    assert metropolis.init_uniform(8, 70, 5).tolist() == g["init_uniform_8x70_seed5"]
    assert metropolis.init_fixed_up(8, 16, 8, 6).tolist() == g["init_fixed_up_8x16_nup8_seed6"]
    c = g["rbm_c1"]
    net = rbm.RBM(np.array(c["W"], np.float32), np.array(c["b"], np.float32), np.array(c["a"], np.float32))
    s, lp, st = metropolis.sweep(net.log_psi, np.array(c["s0"], np.int8), c["nsteps"], seed=c["seed"])
    assert s.tolist() == c["spins"]
    np.testing.assert_allclose(lp, c["log_psi"], rtol=1e-12)


def test_momentum_sr_oracle_limits():
    """The momentum restatements reduce to plain SR where the reference's algebra says so:
    SPRING with mu = 0; MARCH's first step (V = 0 -> no scaling, no momentum yet); AdamSR's
    first step is g + (correction solve) with m_hat = g, so Ebar - Obar m_hat is orthogonal to
    the range used by the second minimum-norm solve and the step equals g for an exact solver."""
    rng = np.random.default_rng(4)
    A = rng.normal(size=(30, 80)) / 9.0
    b = rng.normal(size=30)
    solver = lambda M, v: sr.minnorm_shift(M, v, rshift=0.0, ashift=1e-12)
    g = solver(A, b)
    np.testing.assert_allclose(sr.spring_step(A, b, rng.normal(size=80), 0.0, solver), g, rtol=1e-12, atol=1e-12)
    x, V = sr.march_step(A, b, np.zeros(80), np.zeros(80), 1, 0.95, 0.995, solver, a_dtype=np.float64)
    np.testing.assert_allclose(x, g, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(V, 0.005 * g ** 2, rtol=1e-12)
    x, m, v = sr.adamsr_step(A, b, np.zeros(80), np.zeros(80), 1, 0.95, 0.995, solver, a_dtype=np.float64)
    np.testing.assert_allclose(m, 0.05 * g, rtol=1e-12)
    np.testing.assert_allclose(x, g, rtol=1e-6, atol=1e-6 * np.abs(g).max())


def test_time_evol_oracle_equals_real_time_lstsq():
    """TimeEvol's S-path step equals real-time SR through lstsq_pinv_eig (the same pinv of
    S = Re(Obar^H Obar) applied to -Im(Obar^H Ebar)) on a complex-output state."""
    rng = np.random.default_rng(12)
    O = rng.normal(size=(90, 20)) + 1j * rng.normal(size=(90, 20))
    E = rng.normal(size=90) + 1j * rng.normal(size=90)
    Ob, (eb, _, _) = sr.obar(O), sr.ebar(E)
    S, F = sr.time_evol_sf(Ob, eb)
    x = sr.time_evol_step(S, F, solver=lambda H, b: sr.pinvh(H, b, rtol=1e-9))
    y = sr.solve(Ob, eb, lambda A, b: sr.lstsq_pinv(A, b, rtol=1e-9), complex_out=True, imag_time=False)
    np.testing.assert_allclose(x, y, rtol=1e-10, atol=1e-12)
    assert not np.allclose(x, 0)


def test_rbm_conv_is_the_translated_dense_rbm():
    """The roll-based RBM_Conv equals the dense RBM whose unit (c, x) has the weights
    W_c[(k - x + lo) mod L] (2D 6x4 and a chain of 10), and its log-derivatives match finite
    differences."""
    rng = np.random.default_rng(3)
    for L0, L1 in ((6, 4), (10, 1)):
        C, N = 3, L0 * L1
        W = rng.normal(size=(C, L0, L1)) * 0.3
        b = rng.normal(size=C) * 0.1
        conv = rbm.RBMConv(W, b)
        lo0, lo1 = (L0 - 1) // 2, (L1 - 1) // 2
        Wd = np.zeros((C * N, N))
        for c in range(C):
            for x in range(N):
                for k in range(N):
                    d0 = (k // L1 - x // L1 + lo0) % L0
                    d1 = (k % L1 - x % L1 + lo1) % L1
                    Wd[c * N + x, k] = W[c, d0, d1]
        dense = rbm.RBM(Wd, np.repeat(b, N))
        s = rng.choice([-1.0, 1.0], size=(5, N))
        np.testing.assert_allclose(conv.log_psi(s), dense.log_psi(s), rtol=1e-12)
        J = conv.jacobian(s)
        p = conv.params()
        for k in (0, 7, p.size - 1):
            e = np.zeros_like(p)
            e[k] = 1e-6
            up = rbm.RBMConv((p + e)[:C * N].reshape(C, L0, L1), (p + e)[C * N:])
            dn = rbm.RBMConv((p - e)[:C * N].reshape(C, L0, L1), (p - e)[C * N:])
            np.testing.assert_allclose((up.log_psi(s) - dn.log_psi(s)) / 2e-6, J[:, k], rtol=1e-6, atol=1e-8)


def test_lattices_match_the_reference_code():
    """Site coordinates and n-th nearest-neighbour bonds of the oracle and of the package
    against the output of the reference's own quantax.sites code
    (tests/golden/lattice_reference.json, made by tests/golden/make_lattice_golden.py):
    pins the bond lists the Heisenberg and J1-J2 operators are built from."""
    import json
    from pathlib import Path
    import quantax_gb300 as qtx
    gold = json.loads((Path(__file__).parent / "golden" / "lattice_reference.json").read_text())
    for key, rec in gold.items():
        kind, L = key.split("(")[0], int(key.split("(")[1].rstrip(")"))
        dims = (L,) if kind == "Chain" else (L, L)
        shells = [int(n) for n in rec["neighbors"]]
        ours = lattice.neighbors(dims, shells)
        ours = ours if isinstance(ours, list) else [ours]
        site = getattr(qtx.sites, kind)(L)
        pkg = site.get_neighbor(shells)
        np.testing.assert_allclose(np.asarray(site.coord, dtype=float), np.asarray(rec["coord"]), atol=1e-12)
        for n, o, p in zip(shells, ours, pkg):
            want = np.asarray(rec["neighbors"][str(n)], dtype=np.int64).reshape(-1, 2)
            assert np.array_equal(np.asarray(o), want), (key, n)
            assert np.array_equal(np.asarray(p), want), (key, n)
