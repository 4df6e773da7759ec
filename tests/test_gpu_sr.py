"""GPU parity of the SR / MinSR pieces and of the whole VMC loop against the oracle."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import metropolis, operators as oops, rbm, sr as osr

pytestmark = pytest.mark.gpu


def lib():
    from quantax_gb300 import _lib
    return _lib


def gram(A, mode=0):
    L = lib()
    At = torch.as_tensor(A, dtype=torch.float32).cuda().contiguous()
    n = At.shape[0]
    T = torch.empty((n, n), dtype=torch.float64, device="cuda")
    L.call("qgx_gram", L.ptr(At), n, At.shape[1], At.shape[1], L.ptr(T), n, mode, L.stream_ptr())
    return T.cpu().numpy()


@pytest.mark.parametrize("shape", [(64, 144), (300, 1000), (129, 17), (1, 5), (257, 4100)])
def test_gram_fp32(cuda, shape):
    A = np.random.default_rng(shape[0]).normal(size=shape).astype(np.float32)
    T = gram(A)
    ref = A.astype(np.float64) @ A.astype(np.float64).T
    # FP32 accumulation over k terms: error ~ sqrt(k) eps |a||b|
    tol = 4 * np.sqrt(shape[1]) * 6e-8 * np.sqrt(np.outer(np.diag(ref), np.diag(ref)))
    assert (np.abs(T - ref) <= tol + 1e-30).all()
    assert np.array_equal(T, T.T)


@pytest.mark.parametrize("shape", [(300, 8192), (130, 1000), (1, 7)])
def test_gram_fp64_mode(cuda, shape):
    """QGX_GRAM_FP64: exact FP32 products summed as float pairs, renormalised every 16 terms:
    the Gram of the FP32 matrix to about 1e-13. Stated: 1e-12 of sqrt(T_ii T_jj) per entry
    (FP32 accumulation would be about 1e-6 here)."""
    A = np.random.default_rng(shape[1]).normal(size=shape).astype(np.float32)
    T = gram(A, mode=4)
    ref = A.astype(np.float64) @ A.astype(np.float64).T
    tol = 1e-12 * np.sqrt(np.outer(np.diag(ref), np.diag(ref)))
    assert (np.abs(T - ref) <= tol + 1e-300).all()


def test_gram_transposed(cuda):
    L = lib()
    A = np.random.default_rng(3).normal(size=(500, 130)).astype(np.float32)
    At = torch.as_tensor(A).cuda()
    S = torch.empty((130, 130), dtype=torch.float64, device="cuda")
    L.call("qgx_gram_t", L.ptr(At), 500, 130, 130, L.ptr(S), 130, L.stream_ptr())
    ref = A.astype(np.float64).T @ A.astype(np.float64)
    np.testing.assert_allclose(S.cpu().numpy(), ref, rtol=1e-5, atol=1e-4)


def solve_minsr(A, b, method, **kw):
    L = lib()
    At = torch.as_tensor(A, dtype=torch.float32).cuda()
    bt = torch.as_tensor(b, dtype=torch.float64).cuda()
    n, np_ = A.shape
    T = torch.as_tensor(A.astype(np.float32).astype(np.float64) @ A.astype(np.float32).astype(np.float64).T).cuda()
    nb = C.c_int64(0)
    L.call("qgx_solve_workspace_bytes", n, np_, method, C.byref(nb))
    ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    x = torch.empty(np_, dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    L.call("qgx_minsr_solve", L.ptr(T), n, L.ptr(At), np_, np_, L.ptr(bt), method, kw.get("rshift", 1e-12),
           kw.get("ashift", 1e-4), kw.get("rtol", 1e-12), kw.get("atol", 0.0), kw.get("tol_snr", 0.0), L.ptr(x),
           L.ptr(info), L.ptr(ws), ws.numel(), L.stream_ptr())
    assert int(info.item()) == 0
    return x.cpu().numpy()


@pytest.mark.parametrize("n,np_", [(64, 144), (200, 1000)])
def test_minsr_shift_solve(cuda, n, np_):
    rng = np.random.default_rng(n)
    A = (rng.normal(size=(n, np_)) / np.sqrt(np_)).astype(np.float32)
    b = rng.normal(size=n)
    x = solve_minsr(A, b, 0, ashift=1e-4)
    ref = osr.minnorm_shift(A.astype(np.float64), b, ashift=1e-4)
    np.testing.assert_allclose(x, ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())


@pytest.mark.parametrize("n,np_", [(64, 144), (500, 2000)])
def test_minsr_shift_mixed_solve(cuda, n, np_):
    """FP32 Cholesky + FP64 refinement reaches the FP64 solution (stated: 1e-9 relative;
    the projection x = A^T y accumulates in FP64 like the reference)."""
    rng = np.random.default_rng(n + 1)
    A = (rng.normal(size=(n, np_)) / np.sqrt(np_)).astype(np.float32)
    b = rng.normal(size=n)
    x = solve_minsr(A, b, 2, ashift=1e-4)
    ref = osr.minnorm_shift(A.astype(np.float64), b, ashift=1e-4)
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-9


@pytest.mark.parametrize("tol_snr", [0.0, 0.5])
def test_minsr_pinv_solve(cuda, tol_snr):
    rng = np.random.default_rng(7)
    A = rng.normal(size=(120, 400)).astype(np.float32) / 20
    b = rng.normal(size=120)
    x = solve_minsr(A, b, 1, rtol=1e-12, tol_snr=tol_snr)
    ref = osr.minnorm_pinv(A.astype(np.float64), b, rtol=1e-12, tol_snr=tol_snr)
    np.testing.assert_allclose(x, ref, rtol=1e-6, atol=1e-6 * np.abs(ref).max())


@pytest.mark.parametrize("method", [0, 1])
def test_sr_lstsq_solve(cuda, method):
    L = lib()
    rng = np.random.default_rng(9)
    A = rng.normal(size=(400, 60)).astype(np.float32) / 20
    b = rng.normal(size=400)
    At = torch.as_tensor(A).cuda()
    bt = torch.as_tensor(b).cuda()
    S = torch.empty((60, 60), dtype=torch.float64, device="cuda")
    L.call("qgx_gram_t", L.ptr(At), 400, 60, 60, L.ptr(S), 60, L.stream_ptr())
    nb = C.c_int64(0)
    L.call("qgx_solve_workspace_bytes", 60, 400, method, C.byref(nb))
    ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    x = torch.empty(60, dtype=torch.float64, device="cuda")
    L.call("qgx_sr_solve", L.ptr(S), 60, L.ptr(At), 400, 60, L.ptr(bt), method, 1e-12, 1e-4, 1e-12, 0.0, 0.0,
           L.ptr(x), None, L.ptr(ws), ws.numel(), L.stream_ptr())
    A64 = A.astype(np.float64)
    ref = osr.lstsq_shift(A64, b, ashift=1e-4) if method == 0 else osr.lstsq_pinv(A64, b, rtol=1e-12)
    np.testing.assert_allclose(x.cpu().numpy(), ref, rtol=1e-5, atol=1e-6 * np.abs(ref).max())


@pytest.mark.parametrize("ns,np_,tol_snr", [(400, 60, 0.5), (1000, 130, 2.0), (700, 64, 1.0), (300, 90, 0.0)])
def test_sr_lstsq_pinv_noise_truncation(cuda, ns, np_, tol_snr):
    """lstsq_pinv_eig(tol_snr) on the SR branch (Ns >= Np, solver.py:152-164): the per-sample
    terms b_s (A V)_sk are reduced to their SNR in 64-row chunks; against the oracle's
    _sum_without_noise restatement (stated: 1e-8 relative, FP64 throughout with the FP32 A
    read exactly). Row counts not a multiple of 64 exercise the ragged last chunk."""
    L = lib()
    rng = np.random.default_rng(ns + np_)
    A = (rng.normal(size=(ns, np_)) / 20 + 0.05 * rng.normal(size=(1, np_))).astype(np.float32)
    b = rng.normal(size=ns)
    A64 = A.astype(np.float64)
    S = torch.as_tensor(A64.T @ A64).cuda()
    At, bt = torch.as_tensor(A).cuda(), torch.as_tensor(b).cuda()
    nb = C.c_int64(0)
    L.call("qgx_solve_workspace_bytes", np_, ns, 1, C.byref(nb))
    ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    x = torch.empty(np_, dtype=torch.float64, device="cuda")
    L.call("qgx_sr_solve", L.ptr(S), np_, L.ptr(At), ns, np_, L.ptr(bt), 1, 0.0, 0.0, 1e-12, 0.0, tol_snr,
           L.ptr(x), None, L.ptr(ws), ws.numel(), L.stream_ptr())
    ref = osr.lstsq_pinv(A64, b, rtol=1e-12, tol_snr=tol_snr)
    assert np.linalg.norm(x.cpu().numpy() - ref) < 1e-8 * np.linalg.norm(ref)
    if tol_snr > 0:  # the truncation changes the step: the check is not vacuous
        assert np.linalg.norm(osr.lstsq_pinv(A64, b, rtol=1e-12) - ref) > 1e-3 * np.linalg.norm(ref)


def test_energy_stats(cuda):
    L = lib()
    rng = np.random.default_rng(2)
    E = rng.normal(-10, 1, 1000)
    r = rng.uniform(0.5, 1.5, 1000)
    r /= r.mean()
    Et, rt = torch.as_tensor(E).cuda(), torch.as_tensor(r).cuda()
    stats = torch.empty(3, dtype=torch.float64, device="cuda")
    eb = torch.empty(1000, dtype=torch.float64, device="cuda")
    L.call("qgx_energy_stats", L.ptr(Et), None, L.ptr(rt), 1000, L.ptr(stats), L.ptr(eb), None, L.stream_ptr())
    want_eb, em, var = osr.ebar(E, r)
    s = stats.cpu().numpy()
    assert abs(s[0] - em) < 1e-12 and abs(s[2] - var) < 1e-12 and s[1] == 0.0
    np.testing.assert_allclose(eb.cpu().numpy(), want_eb, rtol=1e-12, atol=1e-14)


def test_update_skips_non_finite(cuda):
    L = lib()
    p = torch.ones(1000, dtype=torch.float32, device="cuda")
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    step = torch.full((1000,), 0.25, dtype=torch.float64, device="cuda")
    L.call("qgx_apply_update", L.ptr(p), L.ptr(step), 1000, L.ptr(flag), L.stream_ptr())
    assert int(flag.item()) == 0 and torch.all(p == 0.75)
    step[123] = float("nan")
    L.call("qgx_apply_update", L.ptr(p), L.ptr(step), 1000, L.ptr(flag), L.stream_ptr())
    assert int(flag.item()) == 1 and torch.all(p == 0.75)


def test_vmc_loop_matches_oracle_and_ed(cuda):
    """Config 1 through the public API: chain L=8 TFIM h=1, RBM M=16 with visible bias,
    64 chains, 16 proposals per sweep, SR with diagonal shift 1e-4, lr 1e-2.

    Every step is checked on identical inputs: the oracle takes the device's parameters,
    runs the same Philox stream from the same configurations (bit-exact samples), and
    computes E_loc, Obar and the SR update in FP64. Stated FP32 tolerances: energy 1e-6
    relative, SR update 1e-3 in relative 2-norm (FP32 Obar / E_loc errors of ~1e-7 are
    amplified by the conditioning of T + 1e-4 I)."""
    import quantax_gb300 as qtx
    qtx.set_random_seed(0)
    qtx.sites.Chain(8)
    H = qtx.operator.Ising(h=1.0)
    W, b, a = rbm.init_normal(8, 16, 0.01, seed=0, visible_bias=True)
    state = qtx.state.Variational(qtx.model.RBM_Dense.from_arrays(W, b, a))
    sampler = qtx.sampler.LocalFlip(state, 64, thermal_steps=0, sweep_steps=16)
    opt = qtx.optimizer.SR(state, H, solver=qtx.optimizer.auto_shift_eig(ashift=1e-4))
    s = sampler.sweep(0).spins.cpu().numpy()
    assert (s == metropolis.init_uniform(64, 8, qtx.global_defs._splitmix64(0 * 0x100000001B3 + 2))).all()
    seed = sampler._seed
    net = rbm.RBM(W, b, a)
    ops = oops.chain_tfim(8)
    step0 = 0
    s, _, _ = metropolis.sweep(net.log_psi, s, 160, seed, step0)
    sampler.sweep(160)
    step0 += 160
    energies, errs = [], []
    for it in range(100):
        if it < 10:
            net.set_params(state.params.cpu().numpy().astype(np.float64))
        samples = sampler.sweep()
        step = opt.get_step(samples)
        energies.append(opt.energy)
        if it < 10:
            s, _, st = metropolis.sweep(net.log_psi, s, 16, seed, step0)
            step0 += 16
            assert (samples.spins.cpu().numpy() == s).all(), f"samples diverged at step {it}"
            E = oops.local_energy(s, ops, net.log_psi).real
            eb, em, var = osr.ebar(E)
            x = osr.solve(osr.obar(net.jacobian(s)), eb, lambda A, b: osr.auto(A, b, "shift", rshift=1e-6, ashift=1e-4))
            assert abs(opt.energy - em) <= 1e-6 * abs(em)
            assert abs(opt.VarE - var) <= 1e-4 * var + 1e-9
            errs.append(np.linalg.norm(step.cpu().numpy() - x) / np.linalg.norm(x))
        state.update(step * 1e-2)
    assert max(errs) < 1e-3, errs
    e_ed = -10.2516617909660
    assert abs(np.mean(energies[-10:]) - e_ed) / abs(e_ed) < 0.02


def _rbm_opt(solver, gram="fp32"):
    import quantax_gb300 as qtx
    qtx.set_default_dtype(np.float64)
    qtx.sites.Chain(8)
    qtx.set_random_seed(1)
    state = qtx.state.Variational(qtx.model.RBM_Dense(16, init_std=0.01))
    return qtx.optimizer.SR(state, qtx.operator.Ising(h=1.0), solver=solver, gram=gram)


@pytest.mark.parametrize("gram,tol", [("fp32", 1e-5), ("3xtf32", 1e-5), ("tf32", 5e-3), ("bf16", 2e-2)])
def test_sr_branch_gram_modes(cuda, gram, tol):
    """Ns >= Np: S = A^T A (tensor-core modes through qgx_transpose) and the shifted solve
    against the FP64 oracle (stated per mode: the operand rounding of the Gram)."""
    import quantax_gb300 as qtx
    opt = _rbm_opt(qtx.optimizer.auto_shift_eig(ashift=1e-3), gram=gram)
    rng = np.random.default_rng(8)
    A = (rng.normal(size=(600, 144)) / 25.0).astype(np.float32)
    b = rng.normal(size=600)
    x = opt.solve(torch.as_tensor(A).cuda(), torch.as_tensor(b).cuda()).cpu().numpy()
    ref = osr.lstsq_shift(A.astype(np.float64), b, rshift=1e-6, ashift=1e-3)
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < tol


def test_mixed_solve_converges_ill_conditioned(cuda):
    """T + shift with condition number ~1e11 (duplicated Obar rows, tiny shift) and a
    right-hand side in the range of Obar: the FP32-preconditioned FP64 conjugate gradients
    converge without falling back, to the FP64 oracle's solution (stated: 1e-6 relative)."""
    import quantax_gb300 as qtx
    opt = _rbm_opt(qtx.optimizer.minnorm_shift_eig(rshift=1e-12, ashift=1e-12, precision="mixed"))
    rng = np.random.default_rng(5)
    Bm = rng.normal(size=(32, 144)) / 12.0
    A = np.concatenate([Bm, Bm]).astype(np.float32)
    c = rng.normal(size=32)
    b = np.concatenate([c, c])  # no component along the near-null directions of T
    x = opt.solve(torch.as_tensor(A).cuda(), torch.as_tensor(b).cuda()).cpu().numpy()
    assert opt.solve_fallbacks == 0
    ref = osr.minnorm_shift(A.astype(np.float64), b, ashift=1e-12)
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-6


def test_mixed_solve_falls_back_to_fp64(cuda):
    """A system the mixed solve cannot finish (condition number ~1e13, right-hand side along
    the near-null directions): it reports info -1, QNGD.solve factors the shifted FP64
    matrix, and the step is exactly that of the FP64 path on the same inputs."""
    import quantax_gb300 as qtx
    rng = np.random.default_rng(6)
    Bm = rng.normal(size=(32, 144)) / 12.0
    A = torch.as_tensor(np.concatenate([Bm, Bm]).astype(np.float32)).cuda()
    b = torch.as_tensor(rng.normal(size=64)).cuda()
    mixed = _rbm_opt(qtx.optimizer.minnorm_shift_eig(rshift=0.0, ashift=1e-13, precision="mixed"))
    x_mixed = mixed.solve(A, b).cpu().numpy()
    assert mixed.solve_fallbacks == 1 and mixed.last_solve_fallback
    plain = _rbm_opt(qtx.optimizer.minnorm_shift_eig(rshift=0.0, ashift=1e-13, precision="fp64"))
    x_fp64 = plain.solve(A, b).cpu().numpy()
    np.testing.assert_array_equal(x_mixed, x_fp64)
