"""The direct samplers (quantax/sampler/sampler.py:14-145): ExactSampler against the oracle's
inverse-CDF draw on the shared Philox stream (bit-exact indices) and against exact energies,
and RandomSampler's configurations and reweight factors."""
import numpy as np
import pytest

from oracle import metropolis, rbm, resconv

pytestmark = pytest.mark.gpu


def _chain_rbm(n=8, M=16, nparticles=None, seed=0):
    import quantax_gb300 as qtx
    qtx.set_default_dtype(np.float64)
    qtx.set_random_seed(seed)
    qtx.sites.Chain(n, Nparticles=nparticles)
    state = qtx.state.Variational(qtx.model.RBM_Dense(M, init_std=0.3, seed=seed))
    p = state.params.cpu().numpy().astype(np.float64)
    return qtx, state, rbm.RBM(p[:M * n].reshape(M, n), p[M * n:])


@pytest.mark.parametrize("reweight", [2.0, 1.0])
def test_exact_sampler_rbm_draws_are_the_oracle_draws(cuda, reweight):
    """Chain(8), all 256 configurations: |psi|^n against the FP64 network (1e-5 relative), the
    drawn basis indices bit-exact against the oracle's inverse CDF on the device's own CDF, two
    sweeps (the Philox step advances), the samples' log psi and reweight factors, and the
    counts of 2^17 draws within 5 standard deviations of N p (bins expecting at least 25;
    the rarer ones pooled)."""
    qtx, state, net = _chain_rbm()
    ns = 1 << 16
    sampler = qtx.sampler.ExactSampler(state, ns, reweight=reweight)
    states = sampler.basis_states
    assert (states == np.arange(256)).all()
    s = qtx.utils.states_to_spins(states, 8).astype(np.float64)
    p, lp = sampler.probabilities()
    x = reweight * net.log_psi(s)
    p_ref = np.exp(x - x.max())
    p_ref /= p_ref.sum()
    np.testing.assert_allclose(p.cpu().numpy(), p_ref, rtol=1e-5)
    counts = np.zeros(256)
    for step in range(2):
        samples = sampler.sweep()
        cdf = sampler._last_cdf.cpu().numpy()
        idx = metropolis.exact_draws(cdf, ns, sampler._seed, step)
        spins = samples.spins.cpu().numpy()
        assert (spins == qtx.utils.states_to_spins(states[idx], 8)).all()
        np.testing.assert_array_equal(samples.log_psi.cpu().numpy(), lp.cpu().numpy()[idx])
        if reweight == 2.0:
            assert samples.reweight_factor is None
        else:
            a = np.exp((2 - reweight) * lp.cpu().numpy()[idx].astype(np.float64))
            np.testing.assert_allclose(samples.reweight_factor.cpu().numpy(), a / a.mean(), rtol=1e-5)
        counts += np.bincount(idx, minlength=256)
    _check_counts(counts, p_ref)


def _check_counts(counts, p):
    expect = p * counts.sum()
    big = expect >= 25
    assert np.all(np.abs(counts[big] - expect[big]) <= 5 * np.sqrt(expect[big]))
    rest, rest_expect = counts[~big].sum(), expect[~big].sum()
    assert abs(rest - rest_expect) <= 5 * np.sqrt(rest_expect) + 5


def test_exact_sampler_energy_matches_exact_reconfiguration(cuda):
    """J1-J2 on 4x4 over the 12870 configurations of Sz = 0, ResConv(2 blocks, 4 channels):
    |psi|^2 against the FP64 network (2e-4 relative), and the mean local energy of 2^15 exact
    samples within 5 standard errors of <psi|H|psi> (ER's energy over the same basis)."""
    import quantax_gb300 as qtx
    qtx.set_default_dtype(np.float64)
    qtx.set_random_seed(4)
    qtx.sites.Square(4, Nparticles=(8, 8))
    H = qtx.operator.Heisenberg(J=[1.0, 0.5], n_neighbor=[1, 2], msr=True)
    state = qtx.state.Variational(qtx.model.ResConv(2, 4, seed=2))
    sampler = qtx.sampler.ExactSampler(state, 1 << 15)
    p, _ = sampler.probabilities()
    s = qtx.utils.states_to_spins(sampler.basis_states, 16).astype(np.float64)
    net = resconv.ResConv(state.params.cpu().numpy(), 4, 2, 4, False)
    x = 2 * np.real(net.log_psi(s))
    p_ref = np.exp(x - x.max())
    p_ref /= p_ref.sum()
    np.testing.assert_allclose(p.cpu().numpy(), p_ref, rtol=2e-4)
    er = qtx.optimizer.ER(state, H)
    er.get_Ebar(er.psi())
    samples = sampler.sweep()
    E = H.Oloc(state, samples).cpu().numpy()
    assert abs(E.mean() - er.energy) <= 5 * E.std() / np.sqrt(len(E))


@pytest.mark.parametrize("nparticles", [None, (8, 8)])
def test_random_sampler(cuda, nparticles):
    """RandomSampler (sampler.py:122-145): configurations uniform over the sector (fixed
    magnetisation when Nparticles is set; site means within 5 standard errors of 0 otherwise),
    log psi equal to the state's, r = |psi|^2 / mean (reweight 0), new draws every sweep."""
    qtx, state, net = _chain_rbm(16, 8, nparticles, seed=1)
    sampler = qtx.sampler.RandomSampler(state, 4096)
    assert sampler.reweight == 0.0
    a = sampler.sweep()
    b = sampler.sweep()
    sa = a.spins.cpu().numpy()
    assert not np.array_equal(sa, b.spins.cpu().numpy())
    if nparticles is None:
        assert np.all(np.abs(sa.mean(axis=0)) <= 5 / np.sqrt(len(sa)))
    else:
        assert (sa.sum(axis=1) == 0).all()
    np.testing.assert_array_equal(a.log_psi.cpu().numpy(), state.log_psi(sa).cpu().numpy())
    lp = net.log_psi(sa.astype(np.float64))
    w = np.exp(2 * (lp - lp.max()))
    np.testing.assert_allclose(a.reweight_factor.cpu().numpy(), w / w.mean(), rtol=1e-4)
