"""Exact reconfiguration (quantax/optimizer/sr.py:432-513) in the full basis against the
reference's reduced basis, on the CPU with the oracle.

The reference sums over the representatives of its symmetry's basis, with psi(rep) / norm(rep)
as coefficients; quantax_gb300.optimizer.ER sums over every configuration of the sector. For
a state projected on the symmetry both give the same energy and the same step: the symmetric
vectors |r> = |orbit|^-1/2 sum_{s in orbit(r)} |s> are orthonormal, psi, H psi and every
d psi / d theta_k lie in their span, so the reduced vectors are the full ones seen through an
isometry. This test builds the reduced basis of the translations of an 8-site chain in the
zero-momentum sector and compares the two computations for a translation-symmetrised RBM."""
import numpy as np

from oracle import operators as oops, rbm, sr as osr


def _sym_rbm(seed=3, M=6, n=8):
    rng = np.random.default_rng(seed)
    net = rbm.RBM(rng.normal(0, 0.3, (M, n)), rng.normal(0, 0.3, M))
    shifts = [np.roll(np.arange(n), -t) for t in range(n)]

    def psi_and_grad(s):
        # psi(s) = mean_g exp(log psi_RBM(T_g s)), d psi = mean_g exp(...) O_RBM(T_g s)
        vals = [np.exp(net.log_psi(s[:, p])) for p in shifts]
        grads = [v[:, None] * net.jacobian(s[:, p]) for v, p in zip(vals, shifts)]
        return np.mean(vals, axis=0), np.mean(grads, axis=0)

    return psi_and_grad


def test_full_and_reduced_basis_give_the_same_step():
    n = 8
    H, states = oops.sparse_matrix(n, oops.chain_tfim(n, 0.7))
    H = H.toarray()
    s = (((states[:, None] >> np.arange(n)) & 1) * 2 - 1)
    psi, dpsi = _sym_rbm()(s)
    # full basis: O = d log psi, as the state's jacobian gives it
    e_f, eb_f, ob_f, _ = osr.er_terms(np.log(psi), dpsi / psi[:, None], H)
    # reduced basis: representatives = smallest code of each translation orbit
    code = lambda x: int(((x > 0).astype(np.int64) << np.arange(n)).sum())
    reps = {}
    for i, x in enumerate(s):
        reps.setdefault(min(code(np.roll(x, t)) for t in range(n)), []).append(i)
    R = sorted(reps)
    U = np.zeros((len(states), len(R)))
    for j, r in enumerate(R):
        members = reps[r]
        U[members, j] = 1.0 / np.sqrt(len(members))
    assert np.allclose(U.T @ U, np.eye(len(R)))
    rep_rows = np.searchsorted(states, R)  # a configuration's code is its basis index
    norm = np.sqrt([len(reps[r]) for r in R])
    c = norm * psi[rep_rows]                      # <r|psi> = |orbit|^1/2 psi(rep)
    O_red = dpsi[rep_rows] / psi[rep_rows, None]  # the jacobian at the representatives
    e_r, eb_r, ob_r, _ = osr.er_terms(np.log(c), O_red, U.T @ H @ U)
    assert abs(e_f - e_r) <= 1e-12 * abs(e_f)
    # the reduced vectors are the full ones through U
    np.testing.assert_allclose(U.T @ eb_f, eb_r, atol=1e-12)
    np.testing.assert_allclose(U.T @ ob_f, ob_r, atol=1e-12)
    np.testing.assert_allclose(ob_f.T @ ob_f, ob_r.T @ ob_r, atol=1e-12)
    for solver in (lambda A, b: osr.auto(A, b, "pinv", rtol=1e-10), lambda A, b: osr.minnorm_pinv(A, b, rtol=1e-10)):
        x_f, x_r = solver(ob_f, eb_f), solver(ob_r, eb_r)
        assert np.linalg.norm(x_f - x_r) <= 1e-8 * np.linalg.norm(x_r)


def test_er_step_lowers_the_energy_to_the_ground_state():
    """ER with an RBM on the 8-site TFIM (h = 1): 100 steps of lr 0.05 from N(0, 0.05^2)
    parameters bring the energy within 1e-5 of the exact ground state (the curve the device
    test follows)."""
    n, M = 8, 16
    rng = np.random.default_rng(0)
    net = rbm.RBM(rng.normal(0, 0.05, (M, n)), rng.normal(0, 0.05, M))
    H, states = oops.sparse_matrix(n, oops.chain_tfim(n, 1.0))
    s = (((states[:, None] >> np.arange(n)) & 1) * 2 - 1)
    E0 = oops.ground_energy(n, oops.chain_tfim(n, 1.0))
    for _ in range(100):
        e, eb, ob, _ = osr.er_terms(net.log_psi(s), net.jacobian(s), H)
        net.set_params(net.params() - 0.05 * osr.auto(ob, eb, "pinv", rtol=1e-6))
    assert abs(e - E0) <= 1e-5 * abs(E0)


def test_exact_draws_follow_the_probabilities():
    """The exact sampler's inverse-CDF draw on the shared Philox stream (oracle/metropolis.py,
    restating jr.choice with p, quantax/sampler/sampler.py:108-110): zero-probability entries
    are never drawn, counts agree with N p, and sweeps draw independently."""
    from oracle import metropolis
    p = np.array([0.0, 0.2, 0.0, 0.05, 0.75, 0.0])
    cdf = np.cumsum(p)
    a = metropolis.exact_draws(cdf, 1 << 16, 123, 0)
    b = metropolis.exact_draws(cdf, 1 << 16, 123, 1)
    assert not np.array_equal(a, b)
    counts = np.bincount(np.concatenate([a, b]), minlength=6)
    assert counts[p == 0].sum() == 0
    expect = p * counts.sum()
    ok = expect > 0
    assert np.all(np.abs(counts[ok] - expect[ok]) <= 5 * np.sqrt(expect[ok]))
    # unnormalised prefix sums give the same draws
    np.testing.assert_array_equal(metropolis.exact_draws(3.0 * cdf, 1 << 16, 123, 0), a)


def test_basis_helpers():
    from math import comb
    from quantax_gb300.utils import basis_states, states_to_spins
    st = basis_states(10, 4)
    assert len(st) == comb(10, 4) and np.all(np.diff(st) > 0)
    s = states_to_spins(st, 10)
    assert s.dtype == np.int8 and np.all((s == 1).sum(axis=1) == 4)
    assert np.array_equal(((s > 0).astype(np.int64) << np.arange(10)).sum(axis=1), st)
    assert len(basis_states(6)) == 64
