"""The no-allocation Obar entry point (qgx_rbm_obar_noalloc) against qgx_rbm_obar.

Callers such as a JAX/XLA FFI custom-call handler or a serving loop with a fixed HBM
budget may not call cudaMalloc; qgx_rbm_obar_noalloc serves them from a static device
array inside the library. This file is collected last so that a run stopping at the
first failure has already run every other test; it also passes on its own in a fresh
process.
"""
import numpy as np
import pytest
import torch

from oracle import metropolis, rbm

pytestmark = pytest.mark.gpu


def _pack(s):
    ns, n = s.shape
    out = np.zeros((ns, (n + 31) // 32), dtype=np.uint32)
    for j in range(n):
        out[:, j // 32] |= (s[:, j] > 0).astype(np.uint32) << np.uint32(j % 32)
    return torch.as_tensor(out.view(np.int32)).cuda()


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


@pytest.mark.parametrize("N,M,ns,vb", [(16, 64, 300, True), (64, 256, 8192, False)])
def test_no_alloc_obar_matches_workspace_entry_on_two_calls(cuda, N, M, ns, vb):
    # two different inputs in a row: the second call must not see the first call's scratch
    for seed in (3, 11):
        table, spins, rt, npar = _case(N, M, ns, vb, seed)
        O_ref, om_ref = _with_workspace(table, N, M, vb, spins, rt, ns, npar)
        O, om = _no_alloc(table, N, M, vb, spins, rt, ns, npar)
        torch.cuda.synchronize()
        # the tolerance of the Obar parity test (tests/test_gpu_rbm.py)
        torch.testing.assert_close(O, O_ref, rtol=1e-4, atol=1e-6 / np.sqrt(ns))
        torch.testing.assert_close(om, om_ref, rtol=1e-5, atol=1e-7)


def test_no_alloc_rejects_requests_beyond_capacity(cuda):
    from quantax_gb300 import _lib as L
    lib = L.lib()
    N, M, ns = 64, 256, 65536  # needs about 200 MB of scratch
    assert lib.qgx_rbm_obar_workspace_bytes(N, M, ns) > (32 << 20)
    rc = lib.qgx_rbm_obar_noalloc(None, N, M, 0, None, None, ns, None, M * N + M, None, None)
    assert rc == L.QGX_ERR_ARG
    assert b"static array" in lib.qgx_last_error()
