"""MixSampler (quantax/sampler/metropolis.py:325-428) of built-in samplers against the oracle's
Metropolis replaying the same component sequence: chains, accepts and log psi."""
import numpy as np
import pytest

from oracle import lattice, metropolis, rbm

pytestmark = pytest.mark.gpu


def test_mix_sampler_bit_exact(cuda):
    import quantax_gb300 as qtx
    from quantax_gb300.state import unpack_spins
    qtx.set_default_dtype(np.float64)
    qtx.set_random_seed(5)
    qtx.sites.Square(4, Nparticles=(8, 8))
    state = qtx.state.Variational(qtx.model.RBM_Dense(24, init_std=0.2, seed=2))
    a = qtx.sampler.SpinExchange(state, 48, thermal_steps=0)
    b = qtx.sampler.SpinExchange(state, 16, thermal_steps=0, n_neighbor=[1, 2])
    c = qtx.sampler.LocalFlip(state, 32, thermal_steps=0)
    mix = qtx.sampler.MixSampler([a, b, c], thermal_steps=0, sweep_steps=60)
    assert mix.nsamples == 96 and mix.nflips == 2
    s0 = unpack_spins(mix._packed, 16).cpu().numpy()
    assert (s0[:48] == unpack_spins(a._packed, 16).cpu().numpy()).all()
    idx = mix.component_sequence(60, 0)
    assert len(set(idx.tolist())) == 3
    samples = mix.sweep()

    p = state.params.cpu().numpy().astype(np.float64)
    net = rbm.RBM(p[:24 * 16].reshape(24, 16), p[24 * 16:])
    tables = [lattice.neighbor_table((4, 4), 1), lattice.neighbor_table((4, 4), [1, 2]), None]
    s, acc, i, margin = s0, np.zeros(96, dtype=np.int64), 0, np.inf
    while i < 60:
        j = i
        while j < 60 and idx[j] == idx[i]:
            j += 1
        t = tables[idx[i]]
        kw = dict(proposal="exchange", nbr_table=t, hop=1) if t is not None else {}
        s, lp, st = metropolis.sweep(net.log_psi, s, j - i, int(mix._seed), i, **kw)
        acc += st["accepts"]
        margin = min(margin, st["min_margin"])
        i = j
    assert margin > 1e-5
    assert (samples.spins.cpu().numpy() == s).all()
    assert (mix.accepts.cpu().numpy() == acc).all()
    np.testing.assert_allclose(samples.log_psi.cpu().numpy(), lp, rtol=2e-6, atol=2e-5)
