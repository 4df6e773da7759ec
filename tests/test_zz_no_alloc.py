"""The no-allocation Obar entry point (qgx_rbm_obar_noalloc) against qgx_rbm_obar.

Callers such as a JAX/XLA FFI custom-call handler or a serving loop with a fixed HBM
budget may not call cudaMalloc; qgx_rbm_obar_noalloc serves them from a static device
array inside the library. Both entry points run the same kernels on the same inputs, so
their outputs must agree bit for bit: any difference means scratch left over from an
earlier call leaked into a result. This file is collected last so that a run stopping at
the first failure has already run every other test; it also passes on its own in a fresh
process.
"""
import numpy as np
import pytest
import torch

from oracle import metropolis, rbm

pytestmark = pytest.mark.gpu

CAPACITY = 32 << 20  # QGX_RBM_OBAR_STATIC_SCRATCH_BYTES


def _pack(s):
    ns, n = s.shape
    out = np.zeros((ns, (n + 31) // 32), dtype=np.uint32)
    for j in range(n):
        out[:, j // 32] |= (s[:, j] > 0).astype(np.uint32) << np.uint32(j % 32)
    return torch.as_tensor(out.view(np.int32)).cuda()


def _largest_ns(lib, N, M):
    """The largest sample count whose scratch fits the static array."""
    lo, hi = 1, 2
    while lib.qgx_rbm_obar_workspace_bytes(N, M, hi) <= CAPACITY:
        lo, hi = hi, 2 * hi
    while hi - lo > 1:
        mid = (lo + hi) // 2
        lo, hi = (mid, hi) if lib.qgx_rbm_obar_workspace_bytes(N, M, mid) <= CAPACITY else (lo, mid)
    return lo


def _case(N, M, ns, vb, seed):
    from quantax_gb300 import _lib as L
    W, b, a = rbm.init_normal(N, M, 0.2, seed=seed, visible_bias=vb)
    Wt = torch.as_tensor(W).cuda()
    bt = torch.as_tensor(b).cuda()
    at = torch.as_tensor(a).cuda() if vb else None
    table = torch.empty(L.lib().qgx_rbm_table_floats(N, M), dtype=torch.float32, device="cuda")
    L.call("qgx_rbm_prepare", L.ptr(Wt), L.ptr(bt), L.ptr(at), N, M, L.ptr(table), L.stream_ptr())
    spins = _pack(metropolis.init_uniform(ns, N, seed + 1))
    r = np.random.default_rng(seed).uniform(0.5, 1.5, ns)
    rt = torch.as_tensor(r / r.mean()).cuda()
    return table, spins, rt, M * N + M + (N if vb else 0)


def _with_workspace(table, N, M, vb, spins, rt, ns, npar):
    from quantax_gb300 import _lib as L
    ws = torch.empty(L.lib().qgx_rbm_obar_workspace_bytes(N, M, ns), dtype=torch.uint8, device="cuda")
    O = torch.empty((ns, npar), dtype=torch.float32, device="cuda")
    om = torch.empty(npar, dtype=torch.float64, device="cuda")
    L.call("qgx_rbm_obar", L.ptr(table), N, M, int(vb), L.ptr(spins), L.ptr(rt), ns, L.ptr(O), npar, L.ptr(om),
           L.ptr(ws), ws.numel(), L.stream_ptr())
    return O, om


def _no_alloc(table, N, M, vb, spins, rt, ns, npar):
    from quantax_gb300 import _lib as L
    O = torch.empty((ns, npar), dtype=torch.float32, device="cuda")
    om = torch.empty(npar, dtype=torch.float64, device="cuda")
    L.call("qgx_rbm_obar_noalloc", L.ptr(table), N, M, int(vb), L.ptr(spins), L.ptr(rt), ns, L.ptr(O), npar,
           L.ptr(om), L.stream_ptr())
    return O, om


def _check_two_calls(N, M, ns, vb):
    # two different inputs in a row: the second call must not see the first call's scratch
    for seed in (3, 11):
        table, spins, rt, npar = _case(N, M, ns, vb, seed)
        O_ref, om_ref = _with_workspace(table, N, M, vb, spins, rt, ns, npar)
        O, om = _no_alloc(table, N, M, vb, spins, rt, ns, npar)
        torch.cuda.synchronize()
        assert torch.equal(O, O_ref), "Obar differs from qgx_rbm_obar"
        assert torch.equal(om, om_ref), "Omean differs from qgx_rbm_obar"


@pytest.mark.parametrize("N,M,ns,vb", [(16, 64, 300, True), (64, 256, 8192, False)])
def test_no_alloc_obar_matches_workspace_entry_on_two_calls(cuda, N, M, ns, vb):
    _check_two_calls(N, M, ns, vb)


def test_no_alloc_at_capacity_and_one_sample_beyond(cuda):
    # the largest request fills the static array to its last byte (16 sites, 64 hidden
    # units: the scratch of 51589 samples is exactly 32 MiB); one sample more is refused
    from quantax_gb300 import _lib as L
    lib = L.lib()
    N, M = 16, 64
    ns = _largest_ns(lib, N, M)
    assert CAPACITY - 4096 < lib.qgx_rbm_obar_workspace_bytes(N, M, ns) <= CAPACITY
    _check_two_calls(N, M, ns, True)
    lib.qgx_clear_last_error()
    rc = lib.qgx_rbm_obar_noalloc(None, N, M, 1, None, None, ns + 1, None, M * N + M + N, None, None)
    assert rc == L.QGX_ERR_ARG
    assert b"static array" in lib.qgx_last_error()


def test_no_alloc_rejects_requests_beyond_capacity(cuda):
    from quantax_gb300 import _lib as L
    lib = L.lib()
    N, M, ns = 64, 256, 65536  # needs about 200 MB of scratch
    assert lib.qgx_rbm_obar_workspace_bytes(N, M, ns) > CAPACITY
    rc = lib.qgx_rbm_obar_noalloc(None, N, M, 0, None, None, ns, None, M * N + M, None, None)
    assert rc == L.QGX_ERR_ARG
    assert b"static array" in lib.qgx_last_error()
    # through the Python binding the refusal carries the library's reason
    with pytest.raises(L.QgxError, match="static array"):
        L.call("qgx_rbm_obar_noalloc", None, N, M, 0, None, None, ns, None, M * N + M, None, None)
