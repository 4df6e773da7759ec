"""Edge cases through the qgx C ABI: empty batches, ragged batch and lattice sizes, and the
largest supported shapes, against the oracle."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import lattice, metropolis, operators as oops, rbm

from test_gpu_rbm import Rbm, pack, unpack, compiled
from test_gpu_resconv import Net, _pack

pytestmark = pytest.mark.gpu


def _lib():
    from quantax_gb300 import _lib
    return _lib


def test_empty_batches_are_no_ops(cuda):
    """ns = 0: every batched entry point returns OK without touching its outputs."""
    L = _lib()
    st = L.stream_ptr()
    W, b, _ = rbm.init_normal(16, 32, 0.1, seed=1)
    dev = Rbm(W, b)
    spins = torch.zeros((1, 1), dtype=torch.int32, device="cuda")
    out = torch.full((4,), 7.0, dtype=torch.float32, device="cuda")
    out64 = torch.full((4,), 7.0, dtype=torch.float64, device="cuda")
    L.call("qgx_rbm_log_psi", L.ptr(dev.table), 16, 32, L.ptr(spins), 0, L.ptr(out), st)
    L.call("qgx_rbm_sweep", L.ptr(dev.table), 16, 32, L.ptr(spins), L.ptr(out), None, 0, 5, 1, 0, 2.0,
           L.PROPOSAL_LOCAL_FLIP, None, 0, 1, st)
    op = compiled(oops.ising_op_list(16, lattice.neighbors((16,), 1), 0.7, 1.0))
    L.call("qgx_rbm_eloc", L.ptr(dev.table), 16, 32, C.byref(op.struct), L.ptr(spins), 0, L.ptr(out64), st)
    net = Net(4, 1, 8, True)
    for prec in (0, 1, 2):
        L.call("qgx_resconv_log_psi", L.ptr(net.table), 4, 1, 8, 1, prec, L.ptr(spins), 0, L.ptr(out), st)
    L.call("qgx_spins_init_uniform", L.ptr(spins), 0, 16, 3, st)
    torch.cuda.synchronize()
    assert torch.equal(out, torch.full((4,), 7.0, device="cuda"))
    assert torch.equal(out64, torch.full((4,), 7.0, dtype=torch.float64, device="cuda"))
    assert int(spins.abs().sum()) == 0


@pytest.mark.parametrize("ns", [1, 33, 257])
def test_ragged_chain_counts_and_word_boundary(cuda, ns):
    """N = 33 sites (two packed words, one bit in the second), chain counts that are not a
    multiple of the warp or block size: LocalFlip bit-exact against the oracle."""
    N, M = 33, 100
    W, b, a = rbm.init_normal(N, M, 0.2, seed=ns, visible_bias=True)
    dev = Rbm(W, b, a)
    net = rbm.RBM(W, b, a)
    s0 = metropolis.init_uniform(ns, N, 5)
    want, want_lp, st = metropolis.sweep(net.log_psi, s0, 40, 9, 0)
    assert st["min_margin"] > 1e-5
    packed = pack(s0)
    lp, acc = dev.sweep(packed, 40, 9)
    assert (unpack(packed, N) == want).all()
    assert (acc.cpu().numpy() == st["accepts"]).all()
    np.testing.assert_allclose(lp.cpu().numpy(), want_lp, rtol=2e-6, atol=2e-5)


@pytest.mark.parametrize("N,M", [(1024, 1024), (200, 600), (256, 513)])
def test_rbm_largest_and_padded_widths(cuda, N, M):
    """N = 1024 sites (32 packed words) and hidden widths padded to 1024 (513 and 600 run with
    zero-weight padding): log psi and a short LocalFlip sweep against the oracle."""
    W, b, _ = rbm.init_normal(N, M, 0.02, seed=N + M)
    dev = Rbm(W, b)
    net = rbm.RBM(W, b)
    s0 = metropolis.init_uniform(16, N, 7)
    packed = pack(s0)
    lp = dev.log_psi(packed).cpu().numpy()
    want = net.log_psi(s0)
    np.testing.assert_allclose(lp, want, rtol=2e-6, atol=2e-4)
    ref, ref_lp, st = metropolis.sweep(net.log_psi, s0, 8, 3, 0)
    assert st["min_margin"] > 1e-4
    lp2, acc = dev.sweep(packed, 8, 3)
    assert (unpack(packed, N) == ref).all()
    assert (acc.cpu().numpy() == st["accepts"]).all()


def test_diagonal_only_operator(cuda):
    """An operator without off-diagonal terms (classical Ising): E_loc is the diagonal energy
    of each configuration, exactly as the oracle computes it."""
    L = _lib()
    N = 20
    ops = [["zz", [[0.8, i, (i + 1) % N] for i in range(N)]], ["z", [[0.3, i] for i in range(N)]]]
    op = compiled(ops)
    W, b, _ = rbm.init_normal(N, 40, 0.1, seed=2)
    dev = Rbm(W, b)
    net = rbm.RBM(W, b)
    s = metropolis.init_uniform(70, N, 4)
    out = torch.empty(70, dtype=torch.float64, device="cuda")
    L.call("qgx_rbm_eloc", L.ptr(dev.table), N, 40, C.byref(op.struct), L.ptr(pack(s)), 70, L.ptr(out),
           L.stream_ptr())
    want = oops.local_energy(s, ops, net.log_psi)
    np.testing.assert_allclose(out.cpu().numpy(), want.real, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("prec,tol", [(0, 3e-4), (1, 5e-3), (2, 4e-2)])
def test_resconv_largest_lattice(cuda, prec, tol):
    """L = 16 (256 sites, the largest supported lattice), 16 channels: log psi against the
    oracle for each convolution arithmetic; one sample and a partly filled CTA."""
    net = Net(16, 2, 16, True, seed=3)
    for ns in (1, 5):
        s = metropolis.init_fixed_up(ns, 256, 128, ns)
        got = net.log_psi(_pack(s), prec)
        want = net.oracle.log_psi(s)
        assert np.abs(got.real - want.real).max() < tol
        assert np.abs(np.angle(np.exp(1j * (got.imag - want.imag)))).max() < tol


def test_resconv_jacobian_largest_lattice(cuda):
    L = _lib()
    net = Net(16, 2, 16, True, seed=4)
    s = metropolis.init_fixed_up(2, 256, 128, 6)
    npar = net.p.size
    O = torch.full((4, npar), float("nan"), dtype=torch.float32, device="cuda")
    ws = torch.empty(L.lib().qgx_resconv_jacobian_workspace_bytes(16, 2, 16), dtype=torch.uint8, device="cuda")
    L.call("qgx_resconv_jacobian", L.ptr(net.table), 16, 2, 16, 1, L.ptr(_pack(s)), 2, L.ptr(O[:2]), L.ptr(O[2:]),
           npar, L.ptr(ws), ws.numel(), L.stream_ptr())
    want = net.oracle.jacobian(s)
    got = O.cpu().numpy().astype(np.float64)
    scale = np.abs(want).max()
    np.testing.assert_allclose(got[:2], want.real, rtol=2e-3, atol=2e-4 * scale)
    np.testing.assert_allclose(got[2:], want.imag, rtol=2e-3, atol=2e-4 * scale)
