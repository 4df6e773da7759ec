"""Real-time evolution: TimeEvol's S-path (quantax/optimizer/time_evol.py:26-134) and real-time
SR (quantax/optimizer/sr.py:90-113) against the oracle, plus the two entry points they add
(qgx_obar_rmatvec, qgx_sym_solve)."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import operators as oops, resconv, sr as osr

pytestmark = pytest.mark.gpu


def _j1j2_state(ns=256):
    import quantax_gb300 as qtx
    qtx.set_random_seed(5)
    qtx.set_default_dtype(np.complex128)
    qtx.sites.Square(4, Nparticles=(8, 8))
    H = qtx.operator.Heisenberg(J=[1.0, 0.5], n_neighbor=[1, 2], msr=True)
    state = qtx.state.Variational(qtx.model.ResConv(2, 8, out_dtype=np.complex64))
    sampler = qtx.sampler.SpinExchange(state, ns, thermal_steps=64, sweep_steps=32)
    return qtx, H, state, sampler


def _oracle_terms(state, samples):
    s = samples.spins.cpu().numpy()
    onet = resconv.ResConv(state.params.cpu().numpy(), 4, 2, 8, True)
    E = oops.local_energy(s, oops.square_j1j2(4, 0.5, True), onet.log_psi)
    eb, em, _ = osr.ebar(E)
    return osr.obar(onet.jacobian(s)), eb, em


def test_time_evol_step_matches_oracle(cuda):
    """J1-J2 on 4x4, ResConv(2 blocks, 8 channels, complex output), 256 SpinExchange samples:
    S, F and the pinvh step against the oracle on identical samples. Stated tolerances: S and F
    within 1e-4 of their largest entry (FP32 network values); the step within 2e-2 relative
    2-norm (the soft inverse cuts eigenvalues below 1e-6 of the largest)."""
    qtx, H, state, sampler = _j1j2_state()
    try:
        opt = qtx.optimizer.TimeEvol(state, H)
        samples = sampler.sweep()
        S, F = opt.get_SF(samples)
        Ob, eb, em = _oracle_terms(state, samples)
        S_ref, F_ref = osr.time_evol_sf(Ob, eb)
        S, F = S.cpu().numpy(), F.cpu().numpy()
        assert np.abs(S - S_ref.real).max() <= 1e-4 * np.abs(S_ref.real).max()
        assert np.abs(F - F_ref).max() <= 1e-4 * np.abs(F_ref).max()
        assert abs(opt.energy - em) <= 1e-5 * abs(em)
        step = opt.get_step(samples).cpu().numpy()
        x = osr.time_evol_step(S_ref, F_ref, solver=lambda M, b: osr.pinvh(M, b, rtol=1e-6))
        assert np.linalg.norm(step - x) / np.linalg.norm(x) < 2e-2
        # the public solve() leaves its arguments alone and repeats get_step's result
        S_dev = torch.as_tensor(S).cuda()
        again = opt.solve(S_dev, torch.as_tensor(F).cuda()).cpu().numpy()
        assert np.array_equal(S_dev.cpu().numpy(), S)
        np.testing.assert_allclose(again, step, rtol=1e-9, atol=1e-12 * np.abs(step).max())
    finally:
        qtx.set_default_dtype(np.float64)


def test_real_time_sr_equals_time_evol(cuda):
    """SR(imag_time=False) through lstsq_pinv_eig solves the same S x = -Im F: the fused
    projection of [-Im; Re] Ebar and TimeEvol's two-pass F agree to rounding."""
    qtx, H, state, sampler = _j1j2_state()
    try:
        samples = sampler.sweep()
        te = qtx.optimizer.TimeEvol(state, H)
        sr = qtx.optimizer.SR(state, H, imag_time=False, solver=qtx.optimizer.lstsq_pinv_eig())
        x1 = te.get_step(samples).cpu().numpy()
        x2 = sr.get_step(samples).cpu().numpy()
        np.testing.assert_allclose(x2, x1, rtol=1e-8, atol=1e-10 * np.abs(x1).max())
        Ob, eb, _ = _oracle_terms(state, samples)
        ref = osr.solve(Ob, eb, lambda A, b: osr.lstsq_pinv(A, b, rtol=1e-6), complex_out=True, imag_time=False)
        assert np.linalg.norm(x2 - ref) / np.linalg.norm(ref) < 2e-2
    finally:
        qtx.set_default_dtype(np.float64)


def test_time_evol_real_state_and_reweight(cuda):
    """A real-output state gets a zero real-time step (the reference's Ebar * 1j); reweighted
    samples are refused with ValueError, as time_evol.py:131-132 does."""
    import quantax_gb300 as qtx
    qtx.set_default_dtype(np.float64)
    qtx.sites.Chain(8)
    qtx.set_random_seed(1)
    state = qtx.state.Variational(qtx.model.RBM_Dense(2, init_std=0.1))
    H = qtx.operator.Ising(h=1.0)
    opt = qtx.optimizer.TimeEvol(state, H)
    samples = qtx.sampler.LocalFlip(state, 64, thermal_steps=16).sweep()
    assert torch.count_nonzero(opt.get_step(samples)) == 0
    rw = qtx.sampler.LocalFlip(state, 64, reweight=1.0, thermal_steps=16).sweep()
    with pytest.raises(ValueError, match="non-reweighted"):
        opt.get_step(rw)


def test_obar_rmatvec_and_sym_solve(cuda):
    from quantax_gb300 import _lib as L
    rng = np.random.default_rng(9)
    rows, cols, lda = 1000, 70, 72
    buf = torch.as_tensor(rng.normal(size=(rows, lda)).astype(np.float32)).cuda()
    A = buf[:, :cols]
    b = rng.normal(size=rows)
    nb = C.c_int64(0)
    L.call("qgx_obar_rmatvec_workspace_bytes", rows, cols, C.byref(nb))
    ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    y = torch.empty(cols, dtype=torch.float64, device="cuda")
    bd = torch.as_tensor(b).cuda()  # held: a temporary's memory could be reused before the launch
    L.call("qgx_obar_rmatvec", L.ptr(A), rows, cols, lda, L.ptr(bd), L.ptr(y), L.ptr(ws), ws.numel(),
           L.stream_ptr())
    An = A.cpu().numpy().astype(np.float64)
    np.testing.assert_allclose(y.cpu().numpy(), An.T @ b, rtol=1e-12, atol=1e-12)

    S = An.T @ An / rows
    f = rng.normal(size=cols)
    for method, ref in ((L.SOLVE_PINV, osr.pinvh(S, f, rtol=1e-9)),
                        (L.SOLVE_SHIFT, np.linalg.solve(S + (1e-6 * np.trace(S) + 1e-3) * np.eye(cols), f))):
        L.call("qgx_solve_workspace_bytes", cols, 1, method, C.byref(nb))
        wss = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
        x = torch.empty(cols, dtype=torch.float64, device="cuda")
        Sd, fd = torch.as_tensor(S).cuda(), torch.as_tensor(f).cuda()
        L.call("qgx_sym_solve", L.ptr(Sd), cols, L.ptr(fd), method, 1e-6, 1e-3, 1e-9, 0.0, L.ptr(x), None,
               L.ptr(wss), wss.numel(), L.stream_ptr())
        np.testing.assert_allclose(x.cpu().numpy(), ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())
