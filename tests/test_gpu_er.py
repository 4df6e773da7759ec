"""Exact reconfiguration (quantax/optimizer/sr.py:432-513) on the GPU against the oracle
(oracle/sr.py er_terms), and the time-stepping drivers (quantax/optimizer/driver.py) against
their restatement from the same device calls."""
import numpy as np
import pytest

from oracle import operators as oops, rbm, resconv, sr as osr

pytestmark = pytest.mark.gpu


def _chain_rbm(M, seed=0, std=0.05):
    import quantax_gb300 as qtx
    qtx.set_default_dtype(np.float64)
    qtx.set_random_seed(seed)
    qtx.sites.Chain(8)
    state = qtx.state.Variational(qtx.model.RBM_Dense(M, init_std=std, seed=seed))
    p = state.params.cpu().numpy().astype(np.float64)
    return qtx, state, rbm.RBM(p[:M * 8].reshape(M, 8), p[M * 8:])


@pytest.mark.parametrize("M", [16, 48])  # Np = 144 < 256 configurations (S branch), 432 > 256 (T branch)
def test_er_rbm_tfim_chain(cuda, M):
    """Chain(8) TFIM (h = 1) over all 256 configurations. Stated: energy 1e-6 relative and Obar
    1e-5 of its largest entry against the FP64 network; Ebar within FP64 rounding of the oracle
    on the device's own amplitudes; the step within 1e-5 of the FP64 pinv (rtol 1e-7) of the
    device's own Obar and Ebar. The Gram is the FP64-class one (about 1e-13 of its largest
    entry); S reaches condition numbers of 2e13 at M = 48, and a 1e-13 perturbation moves the
    pinv step by up to 2e-5 at rtol 1e-9 but below 4e-7 at rtol 1e-7 (measured on the oracle)."""
    qtx, state, net = _chain_rbm(M)
    H = qtx.operator.Ising(h=1.0)
    opt = qtx.optimizer.ER(state, H, solver=qtx.optimizer.auto_pinv_eig(rtol=1e-7))
    Hs, states = oops.sparse_matrix(8, oops.chain_tfim(8, 1.0))
    s = opt.basis_spins.astype(np.float64)
    assert (((states[:, None] >> np.arange(8)) & 1) * 2 - 1 == s).all()
    psi = opt.psi()
    Ebar = opt.get_Ebar(psi)
    Obar = opt.get_Obar(psi)
    e_o, eb_o, ob_o, om_o = osr.er_terms(net.log_psi(s), net.jacobian(s), Hs)
    assert abs(opt.energy - e_o) <= 1e-6 * abs(e_o)
    Ob = Obar.cpu().numpy().astype(np.float64)
    assert np.abs(Ob - ob_o).max() <= 1e-5 * np.abs(ob_o).max()
    np.testing.assert_allclose(opt._Omean.cpu().numpy(), om_o, rtol=0, atol=1e-5 * np.abs(om_o).max())
    lp_dev = state.log_psi_packed(opt._packed).cpu().numpy().astype(np.float64)
    _, eb_d, _, _ = osr.er_terms(lp_dev, np.zeros((len(s), 1)), Hs)
    np.testing.assert_allclose(Ebar.cpu().numpy(), eb_d, rtol=0, atol=1e-12 * np.abs(eb_d).max())
    step = opt.solve(Obar, Ebar).cpu().numpy()
    x = osr.auto(Ob, Ebar.cpu().numpy(), "pinv", rtol=1e-7)
    assert np.linalg.norm(step - x) <= 1e-5 * np.linalg.norm(x)
    # get_step repeats the same sequence of calls
    np.testing.assert_allclose(opt.get_step().cpu().numpy(), step, rtol=0, atol=1e-12 * np.abs(step).max())


def test_er_rbm_reaches_the_ground_state(cuda):
    """100 ER steps of lr 0.05 (default solver) from N(0, 0.05^2) parameters: the FP64 oracle
    run of the same schedule ends within 5e-6 of the exact -10.2516617909660; stated here:
    1e-4 relative (FP32 parameters)."""
    qtx, state, _ = _chain_rbm(16)
    opt = qtx.optimizer.ER(state, qtx.operator.Ising(h=1.0))
    for _ in range(100):
        state.update(0.05 * opt.get_step())
    E0 = oops.ground_energy(8, oops.chain_tfim(8, 1.0))
    assert abs(opt.energy - E0) <= 1e-4 * abs(E0)


def test_er_complex_resconv_j1j2_sector(cuda):
    """J1-J2 (J2 = 0.5, MSR) on 4x4 over the 12870 configurations of Sz = 0, ResConv(2 blocks,
    4 channels, complex output): [Re; Im] Obar rows and Ebar against the oracle on the device's
    own amplitudes and log-derivatives (FP32 Obar storage: 1e-6 of its largest entry), the
    energy against the FP64 network (2e-5 relative), 64 rows of O against the FP64 network, and
    the step against the FP64 pinv of the device's own Obar and Ebar (1e-6)."""
    import quantax_gb300 as qtx
    qtx.set_default_dtype(np.complex128)
    try:
        qtx.sites.Square(4, Nparticles=(8, 8))
        H = qtx.operator.Heisenberg(J=[1.0, 0.5], n_neighbor=[1, 2], msr=True)
        state = qtx.state.Variational(qtx.model.ResConv(2, 4, out_dtype=np.complex64, seed=3))
        opt = qtx.optimizer.ER(state, H, solver=qtx.optimizer.auto_pinv_eig(rtol=1e-9))
        Hs, states = oops.sparse_matrix(16, oops.square_j1j2(4, 0.5, True), nup=8)
        s = opt.basis_spins.astype(np.float64)
        D = len(states)
        assert D == 12870
        psi = opt.psi()
        Ebar = opt.get_Ebar(psi)
        Obar = opt.get_Obar(psi)
        lp = state.log_psi_packed(opt._packed).cpu().numpy().astype(np.complex128)
        O = state.jacobian(opt._packed).cpu().numpy().astype(np.complex128)
        e_d, eb_d, ob_d, om_d = osr.er_terms(lp, O, Hs)
        assert abs(opt.energy - e_d) <= 1e-10 * abs(e_d)
        eb = Ebar.cpu().numpy()
        np.testing.assert_allclose(eb, np.concatenate([eb_d.real, eb_d.imag]), rtol=0,
                                   atol=1e-10 * np.abs(eb_d).max())
        Ob = Obar.cpu().numpy().astype(np.float64)
        ob_ref = np.concatenate([ob_d.real, ob_d.imag])
        assert np.abs(Ob - ob_ref).max() <= 1e-6 * np.abs(ob_ref).max()
        om = opt._Omean.cpu().numpy()
        assert np.abs(om - om_d).max() <= 1e-6 * np.abs(om_d).max()
        net = resconv.ResConv(state.params.cpu().numpy(), 4, 2, 4, True)
        e_net = osr.er_terms(net.log_psi(s), np.zeros((D, 1)), Hs)[0]
        assert abs(opt.energy - e_net) <= 2e-5 * abs(e_net)
        rows = np.random.default_rng(0).choice(D, 64, replace=False)
        O_net = net.jacobian(s[rows])
        assert np.abs(O[rows] - O_net).max() <= 1e-4 * np.abs(O_net).max()
        step = opt.solve(Obar, Ebar).cpu().numpy()
        x = osr.lstsq_pinv(Ob, eb, rtol=1e-9)
        assert np.linalg.norm(step - x) <= 1e-6 * np.linalg.norm(x)
    finally:
        qtx.set_default_dtype(np.float64)


def test_er_rejects_another_symmetry(cuda):
    qtx, state, _ = _chain_rbm(4)
    with pytest.raises(NotImplementedError):
        qtx.optimizer.ER(state, qtx.operator.Ising(h=1.0), symm=qtx.symmetry.TransND())


def test_euler_driver_repeats_the_manual_loop(cuda):
    """Euler (driver.py:30-39) with SR and LocalFlip: three driver steps against three steps of
    sweep / get_step / update on an identically seeded copy; bit-identical parameters and
    traced energies, time = k dt."""
    import quantax_gb300 as qtx

    def build():
        qtx.set_default_dtype(np.float64)
        qtx.set_random_seed(11)
        qtx.sites.Chain(16)
        state = qtx.state.Variational(qtx.model.RBM_Dense(32, init_std=0.05, seed=2))
        sampler = qtx.sampler.LocalFlip(state, 512, thermal_steps=64, sweep_steps=32)
        opt = qtx.optimizer.SR(state, qtx.operator.Ising(h=1.0), solver=qtx.optimizer.auto_shift_eig(ashift=1e-4))
        return state, sampler, opt

    state, sampler, opt = build()
    drv = qtx.optimizer.Euler(state, sampler, opt, 0.02)
    for _ in range(3):
        drv.step()
    p_drv = state.params.cpu().numpy().copy()
    state2, sampler2, opt2 = build()
    energies = []
    for _ in range(3):
        step = opt2.get_step(sampler2.sweep())
        state2.update(0.02 * step)
        energies.append(opt2.energy)
    assert np.array_equal(p_drv, state2.params.cpu().numpy())
    assert np.array_equal(drv.energy.data, np.array(energies))
    np.testing.assert_allclose(drv.energy.time, [0.02, 0.04, 0.06], rtol=1e-12)
    assert len(drv.VarE) == 3 and np.all(drv.VarE.data >= 0)


def test_adaptive_heun_repeats_its_restatement(cuda):
    """AdaptiveHeunEvolution (driver.py:42-104) with TimeEvol on a complex-output ResConv:
    two driver steps against the reference's sequence of sweeps, solves and updates written out
    here on an identically seeded copy, the error estimate sqrt(d^T S d) dt and the clipped
    step-length rule included."""
    import quantax_gb300 as qtx

    def build():
        qtx.set_default_dtype(np.complex128)
        qtx.set_random_seed(5)
        qtx.sites.Square(4, Nparticles=(8, 8))
        H = qtx.operator.Heisenberg(J=[1.0, 0.5], n_neighbor=[1, 2], msr=True)
        state = qtx.state.Variational(qtx.model.ResConv(2, 4, out_dtype=np.complex64, seed=1))
        sampler = qtx.sampler.SpinExchange(state, 256, thermal_steps=64, sweep_steps=16)
        return state, sampler, qtx.optimizer.TimeEvol(state, H)

    try:
        state, sampler, tdvp = build()
        drv = qtx.optimizer.AdaptiveHeunEvolution(state, sampler, tdvp, step_length=2e-3)
        for _ in range(2):
            drv.step()
        p_drv = state.params.cpu().numpy().copy()

        st, sp, td = build()
        dt, t, lengths = 2e-3, 0.0, []
        for _ in range(2):
            si = td.get_step(sp.sweep()); st.update(dt * si)
            sf = td.get_step(sp.sweep()); s1 = (si + sf) / 2; st.update(-dt / 2 * si)
            sm = td.get_step(sp.sweep()); st.update(dt / 4 * (sm - si))
            smm = td.get_step(sp.sweep()); st.update(dt / 2 * smm)
            S, F = td.get_SF(sp.sweep())
            sff = td.solve(S, F); st.update(dt / 4 * (sff - smm))
            d = (s1 - (si + sm + smm + sff) / 4).cpu().numpy()
            err = np.sqrt(d @ S.cpu().numpy() @ d) * dt
            dt = float(np.clip(dt * np.clip((1e-3 / err) ** (1 / 3), 0.2, 2), 1e-4, 1e-2))
            t += dt
            lengths.append(dt)
        np.testing.assert_allclose(p_drv, st.params.cpu().numpy(), rtol=0, atol=1e-6)
        np.testing.assert_allclose(drv.step_size.data, lengths, rtol=1e-9)
        np.testing.assert_allclose(drv.step_size.time, np.cumsum(lengths), rtol=1e-9)
        assert drv.time == pytest.approx(t) and drv.step_length == pytest.approx(dt)
        assert np.isfinite(drv.energy.data).all() and len(drv.VarE) == 2
    finally:
        qtx.set_default_dtype(np.float64)
