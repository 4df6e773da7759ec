"""ResConv forward with the convolutions on the tcgen05 tensor cores (TF32 / BF16 operands,
FP32 accumulation) against the FP64 oracle, through the qgx C ABI.

Stated tolerances (absolute, on Re log psi and on the phase modulo 2 pi; relative on E_loc):
TF32 operands carry 10 explicit mantissa bits and BF16 operands 7, so every convolution
input and weight is rounded with relative error up to 2^-11 resp. 2^-8; through the
residual stack these give the per-precision bounds in TOL_LOGPSI and TOL_ELOC.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import lattice, metropolis, operators as oops

from test_gpu_resconv import Net, _pack, _unpack

pytestmark = pytest.mark.gpu

TF32, BF16 = 1, 2
GROUPED = 0x100  # QGX_CONV_GROUPED
TOL_LOGPSI = {TF32: 5e-3, BF16: 4e-2}
TOL_ELOC = {TF32: 5e-3, BF16: 4e-2}


def _err(got, want):
    dre = np.abs(got.real - want.real).max()
    dph = np.abs(np.angle(np.exp(1j * (got.imag - want.imag)))).max()
    return max(dre, dph)


@pytest.mark.parametrize("prec", [TF32, BF16])
@pytest.mark.parametrize("L,B,Cc,cplx", [(4, 2, 16, True), (10, 8, 16, True), (6, 3, 8, False), (5, 2, 12, True),
                                         (16, 2, 4, True), (3, 1, 16, False)])
def test_resconv_log_psi_tensor_cores(cuda, prec, L, B, Cc, cplx):
    net = Net(L, B, Cc, cplx, seed=L + B)
    n = L * L
    # 300 samples: several CTAs and a partly filled last one
    s = metropolis.init_fixed_up(300, n, n // 2, 3)
    packed = _pack(s)
    want = net.oracle.log_psi(s)
    got = net.log_psi(packed, prec)
    assert _err(got, want) < TOL_LOGPSI[prec], _err(got, want)
    # the FP32 CUDA-core forward is the closer one; both agree to the tensor-core bound
    assert _err(net.log_psi(packed, 0), want) < 2e-4


@pytest.mark.parametrize("prec", [TF32, BF16])
def test_resconv_tensor_core_forward_is_position_independent(cuda, prec):
    """A configuration's log psi does not depend on the batch it is evaluated in (its row
    position in the tiles): the sampler's accept decisions rely on this."""
    net = Net(6, 3, 16, True, seed=4)
    s = metropolis.init_fixed_up(100, 36, 18, 8)
    full = net.log_psi(_pack(s), prec)
    perm = np.random.default_rng(0).permutation(100)
    part = net.log_psi(_pack(s[perm][:37]), prec)
    np.testing.assert_array_equal(part, full[perm][:37])


@pytest.mark.parametrize("prec", [TF32, BF16])
def test_resconv_sweep_tensor_cores_matches_host_replay(cuda, prec):
    """The SpinExchange sweep with the tensor-core forward makes exactly the decisions that
    the oracle's Metropolis loop makes when it is driven by the same forward: identical
    configurations and accept counts on the shared Philox stream."""
    from quantax_gb300 import _lib as Lb
    L, B, Cc, ns = 4, 2, 16, 32
    net = Net(L, B, Cc, True, seed=2, bias_std=0.3)
    n = L * L
    nbr = lattice.neighbor_table((L, L), 1)
    s0 = metropolis.init_fixed_up(ns, n, n // 2, 4)
    seed, nsteps = 77, 24

    def fwd(x):
        return net.log_psi(_pack(np.asarray(x)), prec).real

    want, want_lp, st = metropolis.sweep(fwd, s0, nsteps, seed, 0, proposal="exchange", nbr_table=nbr, hop=1)
    # the device compares in FP32: reweight * (lp' - lp) and log1pf(-u), |log1p(-u)| < 17, are
    # within 2e-6 of the oracle's FP64 values, so decisions agree when every margin is above that
    assert st["min_margin"] > 3e-6
    packed = _pack(s0)
    lp = torch.empty((ns, 2), dtype=torch.float32, device="cuda")
    acc = torch.empty(ns, dtype=torch.int32, device="cuda")
    nbr_t = torch.as_tensor(nbr).cuda()
    ws = torch.empty(Lb.lib().qgx_resconv_sweep_workspace_bytes(L, ns), dtype=torch.uint8, device="cuda")
    Lb.call("qgx_resconv_sweep", Lb.ptr(net.table), L, B, Cc, 1, prec, Lb.ptr(packed), Lb.ptr(lp), Lb.ptr(acc), ns,
            nsteps, seed, 0, 2.0, Lb.ptr(nbr_t), nbr.shape[1], 1, Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    assert (_unpack(packed, n) == want).all()
    assert (acc.cpu().numpy() == st["accepts"]).all()
    np.testing.assert_array_equal(lp.cpu().numpy()[:, 0], want_lp.astype(np.float32))


@pytest.mark.parametrize("prec", [TF32, BF16])
@pytest.mark.parametrize("cplx", [True, False])
def test_resconv_local_energy_tensor_cores(cuda, prec, cplx):
    import quantax_gb300.operator as O
    from quantax_gb300 import _lib as Lb
    L, B, Cc, ns = 6, 3, 16, 64
    net = Net(L, B, Cc, cplx, seed=5)
    n = L * L
    ops = oops.square_j1j2(L, 0.5, True)
    op = O.CompiledOperator(*O.compile_op_list(ops))
    s = metropolis.init_fixed_up(ns, n, n // 2, 9)
    want = oops.local_energy(s, ops, net.oracle.log_psi)
    max_conn = len(op.host["f1"]) + len(op.host["f2"])
    ws = torch.empty(Lb.lib().qgx_resconv_eloc_workspace_bytes(L, ns, max_conn), dtype=torch.uint8, device="cuda")
    er = torch.empty(ns, dtype=torch.float64, device="cuda")
    ei = torch.empty(ns, dtype=torch.float64, device="cuda")
    Lb.call("qgx_resconv_eloc", Lb.ptr(net.table), L, B, Cc, int(cplx), prec, C.byref(op.struct), Lb.ptr(_pack(s)),
            ns, Lb.ptr(er), Lb.ptr(ei), Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    got = er.cpu().numpy() + 1j * ei.cpu().numpy()
    scale = np.abs(want).max()
    assert np.abs(got - want).max() <= TOL_ELOC[prec] * scale, np.abs(got - want).max() / scale


@pytest.mark.parametrize("L,B,Cc,cplx,ns", [(10, 8, 16, True, 16384 + 5), (10, 8, 16, True, 1), (4, 2, 16, True, 300),
                                            (6, 3, 8, False, 1000), (5, 2, 12, True, 777), (8, 6, 16, True, 4096),
                                            (3, 1, 16, False, 50), (16, 2, 4, True, 97)])
def test_bf16_warp_specialised_forward_equals_layer_synchronous(cuda, L, B, Cc, cplx, ns):
    """The warp-specialised BF16 forward (QGX_CONV_GROUPED: sample groups whose epilogues
    overlap the other groups' MMAs, one MMA warp, weights resident) and the default per-layer-
    synchronous kernel run the same arithmetic in the same order: bit-identical log psi for
    every sample count, including a single sample and ragged last groups."""
    net = Net(L, B, Cc, cplx, seed=L + B + 1)
    n = L * L
    packed = _pack(metropolis.init_fixed_up(ns, n, n // 2, 11))
    np.testing.assert_array_equal(net.log_psi(packed, BF16), net.log_psi(packed, BF16 | GROUPED))


def test_bf16_warp_specialised_forward_sinhp1(cuda):
    from quantax_gb300 import _lib as Lb
    net = Net(10, 4, 16, True, seed=3)
    packed = _pack(metropolis.init_fixed_up(2000, 100, 50, 12))
    outs = []
    for prec in (BF16, BF16 | GROUPED):
        out = torch.empty((packed.shape[0], 2), dtype=torch.float32, device="cuda")
        Lb.call("qgx_resconv_log_psi", Lb.ptr(net.table), 10, 4, 16, 1 | 2, prec, Lb.ptr(packed), packed.shape[0],
                Lb.ptr(out), Lb.stream_ptr())
        outs.append(out.cpu().numpy())
    np.testing.assert_array_equal(outs[0], outs[1])
    assert np.isfinite(outs[0]).all()


def test_resconv_tensor_core_arguments(cuda):
    from quantax_gb300 import _lib as Lb
    net = Net(4, 1, 8, True)
    packed = _pack(metropolis.init_fixed_up(4, 16, 8, 1))
    out = torch.empty((4, 2), dtype=torch.float32, device="cuda")
    rc = Lb.lib().qgx_resconv_log_psi(Lb.ptr(net.table), 4, 1, 8, 1, 7, Lb.ptr(packed), 4, Lb.ptr(out), None)
    assert rc == Lb.QGX_ERR_ARG
    # the grouped flag selects a BF16 kernel only
    for prec in (TF32 | GROUPED, GROUPED):
        rc = Lb.lib().qgx_resconv_log_psi(Lb.ptr(net.table), 4, 1, 8, 1, prec, Lb.ptr(packed), 4, Lb.ptr(out), None)
        assert rc == Lb.QGX_ERR_ARG
