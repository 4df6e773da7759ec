"""The FP64 Cholesky factorisation with tensor-core trailing updates (qgx_cholesky) and the
shifted solve built on it (QGX_SOLVE_SHIFT), against LAPACK and cuSOLVER.

Stated bounds: backward error max|L L^T - A| <= 1e-13 max|A| and within 16x of LAPACK's own
factor's; shifted-solve solutions within 1e-9 (relative 2-norm) of cuSOLVER's FP64 Xpotrf path
on well-conditioned Grams; on a matrix of condition number ~6e10 the residual within 8x of
cuSOLVER's and below 1e-12 (the solutions themselves may differ by about cond * 2^-53).
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def lib():
    from quantax_gb300 import _lib
    return _lib


def factor(A):
    L = lib()
    n = A.shape[0]
    At = torch.as_tensor(np.ascontiguousarray(A)).cuda()
    ws = torch.empty(max(L.lib().qgx_cholesky_workspace_bytes(n), 256), dtype=torch.uint8, device="cuda")
    info = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    status = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    L.call("qgx_cholesky", L.ptr(At), n, n, L.ptr(info), L.ptr(status), L.ptr(ws), ws.numel(), L.stream_ptr())
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    return At.cpu().numpy(), int(info.item())


def spd(n, k, seed, shift=1e-4, cond_spread=0.0):
    """T = G G^T + shift I from an FP32 G (the MinSR Gram's structure), optionally with row scales
    spread over exp(N(0, cond_spread))."""
    rng = np.random.default_rng(seed)
    G = rng.normal(size=(n, k)).astype(np.float32).astype(np.float64) / np.sqrt(k)
    if cond_spread:
        G *= np.exp(rng.normal(scale=cond_spread, size=(n, 1)))
    return G @ G.T + shift * np.eye(n)


def backward_error(Lf, A):
    L = np.tril(Lf)
    return np.abs(L @ L.T - A).max() / np.abs(A).max()


@pytest.mark.parametrize("n,k,spread", [(64, 80, 0.0), (100, 150, 0.0), (257, 300, 0.0), (1000, 1200, 1.0),
                                        (2048 + 17, 1500, 0.0), (4096, 4096, 2.0)])
def test_backward_error_against_lapack(cuda, n, k, spread):
    A = spd(n, k, n, cond_spread=spread)
    Lf, info = factor(A)
    assert info == 0
    ours = backward_error(Lf, A)
    ref = backward_error(np.linalg.cholesky(A), A)
    assert ours <= 1e-13, ours
    assert ours <= 16 * ref + 1e-16, (ours, ref)
    # the strict upper triangle is the input's
    iu = np.triu_indices(n, 1)
    assert np.array_equal(Lf[iu], A[iu])


def test_max_digit_panels(cuda):
    """A = L L^T with every below-diagonal entry of L just under a power of two in magnitude:
    the panels' leading digits sit at their bound of 128 and the level sums at their largest."""
    n = 640
    rng = np.random.default_rng(5)
    L0 = np.tril((1.0 - 2.0 ** -9) * np.sign(rng.normal(size=(n, n))), -1) * 2.0 ** -6
    L0[np.diag_indices(n)] = 4.0
    A = L0 @ L0.T
    Lf, info = factor(A)
    assert info == 0
    assert backward_error(Lf, A) <= 1e-14
    assert np.abs(np.tril(Lf) - L0).max() <= 1e-12


@pytest.mark.parametrize("k", [0, 63, 64, 300, 511])
def test_info_reports_first_failing_minor(cuda, k):
    n = 512
    A = spd(n, 600, 11, shift=1e-2)
    A[k, :] = 0.0
    A[:, k] = 0.0
    A[k, k] = -1.0
    _, info = factor(A)
    assert info == k + 1


def _solve(T, A32, b, method):
    L = lib()
    n, np_ = A32.shape
    Tt = torch.as_tensor(T.copy()).cuda()
    At = torch.as_tensor(A32).cuda()
    bt = torch.as_tensor(b).cuda()
    nb = C.c_int64(0)
    L.call("qgx_solve_workspace_bytes", n, np_, method, C.byref(nb))
    ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    x = torch.empty(np_, dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    L.call("qgx_minsr_solve", L.ptr(Tt), n, L.ptr(At), np_, np_, L.ptr(bt), method, 1e-12, 1e-4, 1e-12, 0.0, 0.0,
           L.ptr(x), L.ptr(info), L.ptr(ws), ws.numel(), L.stream_ptr())
    assert int(info.item()) == 0
    return x.cpu().numpy()


@pytest.mark.parametrize("n,np_", [(300, 1000), (2048, 4096), (8192, 8192)])
def test_shift_solve_matches_cusolver(cuda, n, np_):
    from quantax_gb300 import _lib as L
    rng = np.random.default_rng(n)
    A32 = (rng.normal(size=(n, np_)) / np.sqrt(np_)).astype(np.float32)
    A64 = A32.astype(np.float64)
    T = A64 @ A64.T
    b = rng.normal(size=n)
    ours = _solve(T, A32, b, L.SOLVE_SHIFT)
    ref = _solve(T, A32, b, L.SOLVE_SHIFT_LIB)
    assert np.linalg.norm(ours - ref) <= 1e-9 * np.linalg.norm(ref)


def _sym_solve(S, f, method):
    L = lib()
    n = S.shape[0]
    St = torch.as_tensor(S.copy()).cuda()
    ft = torch.as_tensor(f).cuda()
    nb = C.c_int64(0)
    L.call("qgx_solve_workspace_bytes", n, 1, method, C.byref(nb))
    ws = torch.empty(max(nb.value, 256), dtype=torch.uint8, device="cuda")
    y = torch.empty(n, dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    L.call("qgx_sym_solve", L.ptr(St), n, L.ptr(ft), method, 0.0, 0.0, 0.0, 0.0, L.ptr(y), L.ptr(info), L.ptr(ws),
           ws.numel(), L.stream_ptr())
    assert int(info.item()) == 0
    return y.cpu().numpy()


def test_ill_conditioned_shift_solve(cuda):
    """T + 1e-4 I with T a rank-deficient Gram of widely scaled columns (condition number about
    1e10): both factorisations are backward stable, so their solutions may differ by up to
    about cond * 2^-53, but the residuals must be of the same size (stated: within 8x of
    cuSOLVER's, and below 1e-12 relative)."""
    from quantax_gb300 import _lib as L
    n, np_ = 1024, 600
    rng = np.random.default_rng(3)
    A = rng.normal(size=(n, np_)) * np.exp(rng.normal(scale=1.5, size=(1, np_)))
    S = A @ A.T + 1e-4 * np.eye(n)
    w = np.linalg.eigvalsh(S)
    assert w[-1] / w[0] > 1e8
    f = rng.normal(size=n)
    res = {}
    for m in (L.SOLVE_SHIFT, L.SOLVE_SHIFT_LIB):
        y = _sym_solve(S, f, m)
        res[m] = np.linalg.norm(S @ y - f) / (np.linalg.norm(S, 2) * np.linalg.norm(y))
    assert res[L.SOLVE_SHIFT] <= 8 * res[L.SOLVE_SHIFT_LIB] + 1e-16, res
    assert res[L.SOLVE_SHIFT] < 1e-12, res
