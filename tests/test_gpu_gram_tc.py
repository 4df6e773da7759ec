"""tcgen05 Gram matrix (TF32 and BF16 operands, FP32 accumulation) against FP64."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def tc_gram(A, dtype):
    from quantax_gb300 import _lib as L
    At = torch.as_tensor(A, dtype=torch.float32).cuda().contiguous()
    rows, k = At.shape
    src = At
    if dtype == 1:
        src = torch.empty((rows, k), dtype=torch.bfloat16, device="cuda")
        L.call("qgx_f32_to_bf16", L.ptr(At), rows, k, k, L.ptr(src), k, L.stream_ptr())
        assert torch.equal(src, At.to(torch.bfloat16))
    T = torch.full((rows, rows), float("nan"), dtype=torch.float64, device="cuda")
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    L.call("qgx_gram_tc", L.ptr(src), dtype, rows, k, k, L.ptr(T), rows, L.ptr(status), L.stream_ptr())
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    return T.cpu().numpy()


# bound |T - A A^T| <= c ||a_r|| ||a_c||: TF32 keeps 10 mantissa bits, bf16 keeps 7; the
# hi/lo split of FP32 into two TF32 parts keeps ~21 bits per product, and the tensor core's
# FP32 accumulation adds up to ~k 2^-25 on sums of same-sign terms (the diagonal)
TOL = {0: 2.5e-3, 1: 1.0e-2, 2: None}


def tol(dtype, k):
    return TOL[dtype] if TOL[dtype] is not None else 3e-6 + 3e-8 * k


@pytest.mark.parametrize("dtype", [0, 1, 2])
@pytest.mark.parametrize("shape", [(128, 64), (300, 1000), (129, 40), (1024, 4160)])
def test_tc_gram(cuda, dtype, shape):
    A = np.random.default_rng(shape[0] + shape[1]).normal(size=shape).astype(np.float32)
    T = tc_gram(A, dtype)
    A64 = A.astype(np.float64)
    ref = A64 @ A64.T
    d = np.sqrt(np.diag(ref))
    assert np.isfinite(T).all()
    err = np.abs(T - ref) / np.outer(d, d)
    assert err.max() < tol(dtype, shape[1]), err.max()
    # the mirror of every off-diagonal tile is the same accumulator element
    np.testing.assert_allclose(T, T.T, rtol=0, atol=tol(dtype, shape[1]) * np.outer(d, d).max())


def test_tc_gram_through_qgx_gram_mode(cuda):
    from quantax_gb300 import _lib as L
    A = np.random.default_rng(0).normal(size=(256, 512)).astype(np.float32)
    At = torch.as_tensor(A).cuda()
    T = torch.empty((256, 256), dtype=torch.float64, device="cuda")
    L.call("qgx_gram", L.ptr(At), 256, 512, 512, L.ptr(T), 256, L.GRAM_TF32, L.stream_ptr())
    ref = A.astype(np.float64) @ A.astype(np.float64).T
    d = np.sqrt(np.diag(ref))
    assert (np.abs(T.cpu().numpy() - ref) / np.outer(d, d)).max() < TOL[0]


def test_tc_gram_rejects_unaligned_stride(cuda):
    from quantax_gb300 import _lib as L
    A = torch.zeros((64, 30), dtype=torch.float32, device="cuda")
    T = torch.empty((64, 64), dtype=torch.float64, device="cuda")
    rc = L.lib().qgx_gram_tc(L.ptr(A), 0, 64, 30, 30, L.ptr(T), 64, None, L.stream_ptr())
    assert rc == L.QGX_ERR_UNSUPPORTED


def test_tc_gram_long_k_accumulation(cuda):
    """K = 34944 (the ResConv Obar width): the tensor core accumulates 256-element chunks that
    are summed in registers, so the accumulation error does not grow with K (a single FP32
    TMEM accumulator lost ~k 2^-25 = 1e-3 with a systematic sign). Compared with the FP64
    Gram of the same BF16 operands, i.e. accumulation error only (stated: 1e-5)."""
    from quantax_gb300 import _lib as L
    rng = np.random.default_rng(3)
    A = (0.3 * rng.normal(size=34944)[None, :] + rng.normal(size=(256, 34944))).astype(np.float32)
    At = torch.as_tensor(A).cuda()
    Ab = At.to(torch.bfloat16)
    T = torch.empty((256, 256), dtype=torch.float64, device="cuda")
    L.call("qgx_gram_tc", L.ptr(Ab), 1, 256, 34944, 34944, L.ptr(T), 256, None, L.stream_ptr())
    B = Ab.double().cpu().numpy()
    ref = B @ B.T
    d = np.sqrt(np.diag(ref))
    err = np.abs(T.cpu().numpy() - ref) / np.outer(d, d)
    assert err.max() < 1e-5, err.max()


@pytest.mark.parametrize("mode", ["tf32", "bf16", "3xtf32"])
def test_sr_gram_through_transpose(cuda, mode):
    """SR branch (Ns >= Np): S = A^T A as the tensor-core Gram of A^T (qgx_transpose)."""
    from quantax_gb300 import _lib as L
    ns, np_ = 2000, 300
    A = np.random.default_rng(9).normal(size=(ns, np_)).astype(np.float32)
    At = torch.as_tensor(A).cuda()
    ld = (ns + 7) // 8 * 8
    bf16 = mode == "bf16"
    Atr = torch.empty((np_, ld), dtype=torch.bfloat16 if bf16 else torch.float32, device="cuda")
    L.call("qgx_transpose", L.ptr(At), ns, np_, np_, L.ptr(Atr), ld, int(bf16), L.stream_ptr())
    if bf16:
        assert torch.equal(Atr[:, :ns], At.t().to(torch.bfloat16))
    else:
        assert torch.equal(Atr[:, :ns], At.t())
    S = torch.empty((np_, np_), dtype=torch.float64, device="cuda")
    if bf16:
        L.call("qgx_gram_tc", L.ptr(Atr), 1, np_, ns, ld, L.ptr(S), np_, None, L.stream_ptr())
    else:
        m = {"tf32": L.GRAM_TF32, "3xtf32": L.GRAM_3XTF32}[mode]
        L.call("qgx_gram", L.ptr(Atr), np_, ns, ld, L.ptr(S), np_, m, L.stream_ptr())
    ref = A.astype(np.float64).T @ A.astype(np.float64)
    d = np.sqrt(np.diag(ref))
    err = np.abs(S.cpu().numpy() - ref) / np.outer(d, d)
    assert err.max() < tol({"tf32": 0, "bf16": 1, "3xtf32": 2}[mode], ns), err.max()


def _tf32(a, round_half=False):
    """The TF32 value of FP32 entries: truncated (13 low mantissa bits cleared) or, with
    round_half, rounded half away from zero on the 13th bit."""
    bits = np.asarray(a, dtype=np.float32).view(np.uint32)
    if round_half:
        bits = bits + np.uint32(0x1000)
    return (bits & np.uint32(0xFFFFE000)).view(np.float32)


def test_tf32_operands_are_truncated(cuda):
    """The split-TF32 Gram uses the staged FP32 operand itself as its high part, relying on the
    tensor core reading an FP32 operand as TF32 by ignoring its 13 low mantissa bits. A TF32
    Gram of raw operands and one of operands truncated on the host agree bit for bit, while
    operands rounded on the host give a different result (the check has teeth)."""
    A = np.random.default_rng(21).normal(size=(256, 512)).astype(np.float32)
    T_raw = tc_gram(A, 0)
    assert np.array_equal(T_raw, tc_gram(_tf32(A), 0))
    assert not np.array_equal(T_raw, tc_gram(_tf32(A, round_half=True), 0))


@pytest.mark.parametrize("shape", [(256, 512), (300, 1000)])
def test_split_tf32_gram_is_its_three_products(cuda, shape):
    """3xtf32 computes hi hi^T + hi lo^T + lo hi^T with hi = tf32(x) and lo = tf32(x - hi), the
    values the tensor core reads. Against that sum in FP64, only the FP32 accumulation of
    256-element chunks remains, stated in units of |a_r| |a_c|: 1e-6 off the diagonal (measured
    below 1e-7) and the accumulation bound of the other tests on it, where the same-sign sums
    lose up to an FP32 ulp per MMA (measured 5.5e-6 at k = 512). A wrong high part would show
    TF32-size errors: 2^-11 / sqrt(k) = 2e-5 off the diagonal at k = 512, 2^-11 = 5e-4 on it."""
    A = np.random.default_rng(shape[0]).normal(size=shape).astype(np.float32)
    hi = _tf32(A)
    lo = _tf32(A - hi)
    h, l = hi.astype(np.float64), lo.astype(np.float64)
    ref = h @ h.T + h @ l.T + l @ h.T
    T = tc_gram(A, 2)
    d = np.linalg.norm(A.astype(np.float64), axis=1)
    err = np.abs(T - ref) / np.outer(d, d)
    off = ~np.eye(shape[0], dtype=bool)
    assert err[off].max() < 1e-6, err[off].max()
    assert np.diag(err).max() < tol(2, shape[1]), np.diag(err).max()
