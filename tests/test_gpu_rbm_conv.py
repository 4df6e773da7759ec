"""RBM_Conv (quantax/model/shallow_nets.py:129-190) on the GPU against the roll-based oracle
(oracle/rbm.py RBMConv): log psi, the Metropolis sweep (bit-exact decisions), local energies,
log-derivatives, and one SR step of the examples/RBM.ipynb workload shape. The 10 x 10 lattice
with 16 channels is 1600 hidden units, the 2048-wide kernels."""

import numpy as np
import pytest
import torch

from oracle import lattice, metropolis, operators as oops, rbm, sr as osr

pytestmark = pytest.mark.gpu


def _state(dims, channels, std=0.05, seed=3):
    import quantax_gb300 as qtx
    qtx.set_default_dtype(np.float64)
    qtx.set_random_seed(seed)
    if len(dims) == 1:
        qtx.sites.Chain(dims[0], Nparticles=(dims[0] // 2, dims[0] // 2))
    else:
        qtx.sites.Square(dims[0], Nparticles=(dims[0] ** 2 // 2, dims[0] ** 2 // 2))
    model = qtx.model.RBM_Conv(channels, init_std=std, seed=seed)
    state = qtx.state.Variational(model)
    p = state.params.cpu().numpy().astype(np.float64)
    L0 = dims[0]
    L1 = dims[1] if len(dims) > 1 else 1
    N = L0 * L1
    net = rbm.RBMConv(p[:channels * N].reshape(channels, L0, L1), p[channels * N:])
    return qtx, state, net


@pytest.mark.parametrize("dims,channels", [((16,), 4), ((6, 6), 8), ((10, 10), 16)])
def test_rbm_conv_log_psi_and_jacobian(cuda, dims, channels):
    qtx, state, net = _state(dims, channels)
    n = int(np.prod(dims))
    s = metropolis.init_fixed_up(24, n, n // 2, 5)
    got = state.log_psi(s).cpu().numpy()
    want = net.log_psi(s)
    # FP32 sum of channels x N log-cosh terms
    np.testing.assert_allclose(got, want, rtol=0, atol=2e-6 * channels * n + 1e-5)
    O = state.jacobian(s).cpu().numpy()
    Ow = net.jacobian(s)
    np.testing.assert_allclose(O, Ow, rtol=1e-4, atol=1e-5 * np.abs(Ow).max())


@pytest.mark.parametrize("dims,channels,prop", [((16,), 4, "flip"), ((6, 6), 8, "exchange"),
                                                ((10, 10), 16, "exchange")])
def test_rbm_conv_sweep_bit_exact(cuda, dims, channels, prop):
    from quantax_gb300 import _lib as L
    qtx, state, net = _state(dims, channels, std=0.1, seed=7)
    n = int(np.prod(dims))
    ns, nsteps, seed = 32, 40, 123
    s0 = metropolis.init_fixed_up(ns, n, n // 2, 2)
    if prop == "exchange":
        nbr = lattice.neighbor_table(dims, 1)
        want, want_lp, st = metropolis.sweep(net.log_psi, s0, nsteps, seed, 0, proposal="exchange", nbr_table=nbr,
                                             hop=1)
        code, nbr_t, z = L.PROPOSAL_SPIN_EXCHANGE, torch.as_tensor(nbr).cuda(), nbr.shape[1]
    else:
        want, want_lp, st = metropolis.sweep(net.log_psi, s0, nsteps, seed, 0)
        code, nbr_t, z = L.PROPOSAL_LOCAL_FLIP, None, 0
    assert st["min_margin"] > 1e-5
    from quantax_gb300.state import pack_spins, unpack_spins
    packed = pack_spins(s0, n)
    lp = torch.empty(ns, dtype=torch.float32, device="cuda")
    acc = torch.empty(ns, dtype=torch.int32, device="cuda")
    L.call("qgx_rbm_sweep", L.ptr(state.table), n, channels * n, L.ptr(packed), L.ptr(lp), L.ptr(acc), ns, nsteps,
           seed, 0, 2.0, code, L.ptr(nbr_t), z, 1, L.stream_ptr())
    assert (unpack_spins(packed, n).cpu().numpy() == want).all()
    assert (acc.cpu().numpy() == st["accepts"]).all()
    np.testing.assert_allclose(lp.cpu().numpy(), want_lp, rtol=0, atol=2e-6 * channels * n + 1e-5)


def test_rbm_conv_sr_step(cuda):
    """examples/RBM.ipynb's setup at a test size: 10 x 10 Heisenberg (MSR), RBM_Conv(16),
    SpinExchange, SR with lstsq_pinv_eig(rtol=1e-9) (Ns >= Np: the S = Obar^T Obar branch).
    rtol = 1e-9 keeps eigenvalues far below FP32 resolution, so S is the FP64 Gram
    (gram="fp64") of the FP32 Obar. Stated: E_loc 1e-5 of max |E_loc|, energy 1e-6 relative,
    Obar 1e-4 of its largest entry against the FP64 oracle; the update within 1e-6 of the FP64
    solve of the device's own Obar (the pinv of a matrix whose condition number reaches 1e9
    magnifies the 1e-7 differences between FP32 and FP64 network values, so the update is
    compared on the same Obar)."""
    qtx, state, net = _state((10, 10), 16, std=0.02, seed=1)
    H = qtx.operator.Heisenberg(msr=True)
    sampler = qtx.sampler.SpinExchange(state, 2048, thermal_steps=100, sweep_steps=50)
    opt = qtx.optimizer.SR(state, H, solver=qtx.optimizer.lstsq_pinv_eig(rtol=1e-9), gram="fp64")
    samples = sampler.sweep()
    s = samples.spins.cpu().numpy()
    E_dev = H.Oloc(state, samples).cpu().numpy()
    ops = oops.heisenberg_op_list(lattice.neighbors((10, 10), [1]), [1.0], [1], True)
    E = oops.local_energy(s, ops, net.log_psi).real
    np.testing.assert_allclose(E_dev, E, rtol=0, atol=1e-5 * np.abs(E).max())
    Ebar = opt.get_Ebar(samples)
    Obar = opt.get_Obar(samples)
    Ob_dev = Obar.cpu().numpy().astype(np.float64)
    eb_dev = Ebar.cpu().numpy()
    step = opt.solve(Obar, Ebar).cpu().numpy()
    eb, em, _ = osr.ebar(E)
    Ob = osr.obar(net.jacobian(s))
    assert abs(opt.energy - em) <= 1e-6 * abs(em)
    assert np.abs(Ob_dev - Ob).max() <= 1e-4 * np.abs(Ob).max()
    x = osr.lstsq_pinv(Ob_dev, eb_dev, rtol=1e-9)
    assert np.linalg.norm(step - x) / np.linalg.norm(x) < 1e-6
