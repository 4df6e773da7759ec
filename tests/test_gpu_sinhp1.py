"""ResConv with the sinhp1_by_scale final activation (quantax/nn/activation.py:7-15), the J1-J2
notebook's model: psi = mean (sinh z + 1), negative on part of the configurations for a real
output. Forward (FP32, TF32, BF16), E_loc, log-derivatives and the sweep against the oracle.

Stated tolerances: as the exp_by_scale tests (log psi 2e-4 FP32, 5e-3 TF32, 4e-2 BF16) times
kappa = mean |sinh z + 1| / |mean (sinh z + 1)|, the amplification of a mean that cancels."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import lattice, metropolis, operators as oops, resconv

from test_gpu_resconv import _pack, _unpack

pytestmark = pytest.mark.gpu

SINHP1 = 2


class Net:
    def __init__(self, L, B, Cc, cplx, seed=0, bias_std=0.1, shift=0.0):
        """shift: added to block 0's second biases, which moves the features down so that the
        mean of sinh z + 1 changes sign across configurations (-1.2 at 4x4, 2 blocks, 8
        channels, seed 6: about a quarter of them negative)."""
        from quantax_gb300 import _lib as Lb
        self.L, self.B, self.C, self.cplx = L, B, Cc, cplx
        self.flags = int(cplx) | SINHP1
        self.p = resconv.init_he(B, Cc, seed=seed, bias_std=bias_std)
        o = Cc * 9 + Cc + Cc * Cc * 9  # block 0: conv1 weights and biases, conv2 weights
        if B > 1:
            self.p[o:o + Cc] += shift
        self.pt = torch.as_tensor(self.p).cuda()
        self.table = torch.empty(Lb.lib().qgx_resconv_table_floats(B, Cc), dtype=torch.float32, device="cuda")
        Lb.call("qgx_resconv_prepare", Lb.ptr(self.pt), B, Cc, Lb.ptr(self.table), Lb.stream_ptr())
        self.oracle = resconv.ResConv(self.p, L, B, Cc, cplx, sinhp1=True)

    def log_psi(self, s, prec=0):
        from quantax_gb300 import _lib as Lb
        packed = _pack(s)
        out = torch.empty((s.shape[0], 2), dtype=torch.float32, device="cuda")
        Lb.call("qgx_resconv_log_psi", Lb.ptr(self.table), self.L, self.B, self.C, self.flags, prec, Lb.ptr(packed),
                s.shape[0], Lb.ptr(out), Lb.stream_ptr())
        o = out.cpu().numpy().astype(np.float64)
        return o[:, 0] + 1j * o[:, 1]

    def kappa(self, s):
        x = resconv.features(torch.as_tensor(self.p, dtype=torch.float64), torch.as_tensor(s, dtype=torch.float64),
                             self.L, self.B, self.C).numpy().reshape(s.shape[0], -1)
        if self.cplx:
            c2 = x.shape[1] // 2
            x = x[:, :c2] + 1j * x[:, c2:]
        f = np.sinh(x) + 1
        return np.abs(f).mean(axis=1) / np.abs(f.mean(axis=1))


def _check_logpsi(got, want, tol, kappa):
    assert (np.abs(got.real - want.real) <= tol * kappa).all()
    assert (np.abs(np.angle(np.exp(1j * (got.imag - want.imag)))) <= tol * kappa).all()


@pytest.mark.parametrize("L,B,Cc,cplx", [(4, 2, 8, False), (4, 2, 8, True), (10, 4, 16, False), (6, 3, 12, True)])
@pytest.mark.parametrize("prec,tol", [(0, 2e-4), (1, 5e-3), (2, 4e-2)])
def test_sinhp1_log_psi(cuda, L, B, Cc, cplx, prec, tol):
    signed = not cplx and L == 4
    net = Net(L, B, Cc, cplx, seed=6 if signed else L + B, bias_std=0.3, shift=-1.2 if signed else 0.0)
    n = L * L
    s = metropolis.init_fixed_up(40, n, n // 2, 3)
    want = net.oracle.log_psi(s)
    _check_logpsi(net.log_psi(s, prec), want, tol, net.kappa(s))
    if signed:
        ph = np.abs(np.angle(np.exp(1j * want.imag)))
        assert (ph > 1).any() and (ph < 1).any(), "the test wants amplitudes of both signs"


@pytest.mark.parametrize("cplx", [False, True])
def test_sinhp1_local_energy(cuda, cplx):
    import quantax_gb300.operator as O
    from quantax_gb300 import _lib as Lb
    L = 4
    net = Net(L, 2, 8, cplx, seed=6, bias_std=0.3, shift=0.0 if cplx else -1.2)
    ops = oops.square_j1j2(L, 0.5, True)
    op = O.CompiledOperator(*O.compile_op_list(ops))
    pool = metropolis.init_fixed_up(200, 16, 8, 9)
    s = pool[net.kappa(pool) < 30][:40]  # configurations a chain visits: psi not cancelling
    assert s.shape[0] == 40
    want = oops.local_energy(s, ops, net.oracle.log_psi)
    max_conn = len(op.host["f1"]) + len(op.host["f2"])
    ws = torch.empty(Lb.lib().qgx_resconv_eloc_workspace_bytes(L, 40, max_conn), dtype=torch.uint8, device="cuda")
    er = torch.empty(40, dtype=torch.float64, device="cuda")
    ei = torch.empty(40, dtype=torch.float64, device="cuda")
    packed = _pack(s)
    Lb.call("qgx_resconv_eloc", Lb.ptr(net.table), L, 2, 8, net.flags, 0, C.byref(op.struct), Lb.ptr(packed), 40,
            Lb.ptr(er), Lb.ptr(ei), Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    got = er.cpu().numpy() + 1j * ei.cpu().numpy()
    if not cplx:
        got, want = got.real, want.real
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-3 * np.abs(want).max())


@pytest.mark.parametrize("L,B,Cc,cplx", [(4, 2, 8, False), (4, 2, 8, True), (6, 3, 4, False)])
def test_sinhp1_jacobian(cuda, L, B, Cc, cplx):
    from quantax_gb300 import _lib as Lb
    signed = not cplx and (L, B, Cc) == (4, 2, 8)
    net = Net(L, B, Cc, cplx, seed=6 if signed else 7, bias_std=0.3, shift=-1.2 if signed else 0.0)
    n = L * L
    pool = metropolis.init_fixed_up(60, n, n // 2, 2)
    s = pool[net.kappa(pool) < 30][:6]
    ns = s.shape[0]
    assert ns == 6
    npar = net.p.size
    O = torch.full((2 * ns, npar), float("nan"), dtype=torch.float32, device="cuda")
    ws = torch.empty(Lb.lib().qgx_resconv_jacobian_workspace_bytes(L, B, Cc), dtype=torch.uint8, device="cuda")
    packed = _pack(s)
    Lb.call("qgx_resconv_jacobian", Lb.ptr(net.table), L, B, Cc, net.flags, Lb.ptr(packed), ns, Lb.ptr(O[:ns]),
            Lb.ptr(O[ns:]) if cplx else None, npar, Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    want = net.oracle.jacobian(s)
    got = O.cpu().numpy().astype(np.float64)
    kappa = net.kappa(s)[:, None]
    bound = (2e-3 * np.abs(want) + 2e-4 * np.abs(want).max()) * kappa
    assert (np.abs(got[:ns] - want.real) <= bound).all()
    if cplx:
        assert (np.abs(got[ns:] - want.imag) <= bound).all()


def test_sinhp1_sweep_bit_exact(cuda):
    from quantax_gb300 import _lib as Lb
    L, ns, seed, nsteps = 4, 32, 91, 24
    net = Net(L, 2, 8, False, seed=2, bias_std=0.3)
    nbr = lattice.neighbor_table((L, L), 1)
    s0 = metropolis.init_fixed_up(ns, 16, 8, 4)
    want, want_lp, st = metropolis.sweep(lambda x: net.oracle.log_psi(x).real, s0, nsteps, seed, 0,
                                         proposal="exchange", nbr_table=nbr, hop=1)
    assert st["min_margin"] > 1e-4
    packed = _pack(s0)
    lp = torch.empty((ns, 2), dtype=torch.float32, device="cuda")
    acc = torch.empty(ns, dtype=torch.int32, device="cuda")
    nbr_t = torch.as_tensor(nbr).cuda()
    ws = torch.empty(Lb.lib().qgx_resconv_sweep_workspace_bytes(L, ns), dtype=torch.uint8, device="cuda")
    Lb.call("qgx_resconv_sweep", Lb.ptr(net.table), L, 2, 8, net.flags, 0, Lb.ptr(packed), Lb.ptr(lp), Lb.ptr(acc),
            ns, nsteps, seed, 0, 2.0, Lb.ptr(nbr_t), nbr.shape[1], 1, Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    assert (_unpack(packed, 16) == want).all()
    assert (acc.cpu().numpy() == st["accepts"]).all()


def test_sinhp1_state_api(cuda):
    """ResConv(final_activation=qtx.nn.sinhp1_by_scale) through the public API: a real state
    whose log psi is complex (phase 0 or pi) and psi(s) real with both signs."""
    import quantax_gb300 as qtx
    qtx.set_random_seed(4)
    qtx.set_default_dtype(np.float64)
    qtx.sites.Square(4, Nparticles=(8, 8))
    model = qtx.model.ResConv(2, 8, final_activation=qtx.nn.sinhp1_by_scale)
    state = qtx.state.Variational(model)
    s = metropolis.init_fixed_up(64, 16, 8, 1)
    lp = state.log_psi(s)
    assert lp.is_complex()
    onet = resconv.ResConv(state.params.cpu().numpy(), 4, 2, 8, False, sinhp1=True)
    psi = state(s).cpu().numpy()
    want = np.exp(onet.log_psi(s)).real
    assert not np.iscomplexobj(psi)
    np.testing.assert_allclose(psi, want, rtol=2e-3, atol=1e-3 * np.abs(want).max())
