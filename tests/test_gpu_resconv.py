"""GPU parity of the ResConv kernels against the FP64 oracle, through the qgx C ABI."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import lattice, metropolis, operators as oops, resconv

pytestmark = pytest.mark.gpu


def _pack(s):
    ns, n = s.shape
    out = np.zeros((ns, (n + 31) // 32), dtype=np.uint32)
    for j in range(n):
        out[:, j // 32] |= (s[:, j] > 0).astype(np.uint32) << np.uint32(j % 32)
    return torch.as_tensor(out.view(np.int32)).cuda()


def _unpack(t, n):
    w = t.cpu().numpy().view(np.uint32)
    out = np.empty((w.shape[0], n), dtype=np.int8)
    for j in range(n):
        out[:, j] = ((w[:, j // 32] >> np.uint32(j % 32)) & 1).astype(np.int8) * 2 - 1
    return out


class Net:
    def __init__(self, L, B, Cc, cplx, seed=0, bias_std=0.1):
        from quantax_gb300 import _lib as Lb
        self.L, self.B, self.C, self.cplx = L, B, Cc, cplx
        self.p = resconv.init_he(B, Cc, seed=seed, bias_std=bias_std)
        assert Lb.lib().qgx_resconv_nparams(B, Cc) == self.p.size
        self.pt = torch.as_tensor(self.p).cuda()
        self.table = torch.empty(Lb.lib().qgx_resconv_table_floats(B, Cc), dtype=torch.float32, device="cuda")
        Lb.call("qgx_resconv_prepare", Lb.ptr(self.pt), B, Cc, Lb.ptr(self.table), Lb.stream_ptr())
        self.oracle = resconv.ResConv(self.p, L, B, Cc, cplx)

    def log_psi(self, packed, prec=0):
        from quantax_gb300 import _lib as Lb
        out = torch.empty((packed.shape[0], 2), dtype=torch.float32, device="cuda")
        Lb.call("qgx_resconv_log_psi", Lb.ptr(self.table), self.L, self.B, self.C, int(self.cplx), prec,
                Lb.ptr(packed), packed.shape[0], Lb.ptr(out), Lb.stream_ptr())
        o = out.cpu().numpy().astype(np.float64)
        return o[:, 0] + 1j * o[:, 1]


def _close_logpsi(got, want, tol):
    # phases compared modulo 2 pi
    assert np.abs(got.real - want.real).max() < tol
    dph = np.angle(np.exp(1j * (got.imag - want.imag)))
    assert np.abs(dph).max() < tol


@pytest.mark.parametrize("L,B,Cc,cplx", [(4, 2, 8, True), (6, 3, 4, False), (10, 8, 16, True), (5, 1, 12, True)])
def test_resconv_log_psi(cuda, L, B, Cc, cplx):
    net = Net(L, B, Cc, cplx, seed=L + B)
    n = L * L
    s = metropolis.init_fixed_up(37, n, n // 2, 3)
    _close_logpsi(net.log_psi(_pack(s)), net.oracle.log_psi(s), 2e-4)


@pytest.mark.parametrize("L,Cc,cplx", [(4, 8, True), (6, 8, False), (4, 4, True)])
def test_fp32_forward_orders_agree_bitwise(cuda, L, Cc, cplx):
    """Below 12 channels the FP32 forward keeps the site order for a batch that cannot give every
    SM two CTAs, and takes the blocked order (2 x 2 site blocks) once it can. The same 512
    configurations alone (site order) and inside a batch of 32768 (blocked order) must give the
    same floats."""
    net = Net(L, 2, Cc, cplx, seed=6, bias_std=0.2)
    s = metropolis.init_uniform(512, L * L, 3)
    small = net.log_psi(_pack(s))
    big = net.log_psi(_pack(np.tile(s, (64, 1))))
    assert np.array_equal(small, big[:512])
    assert np.array_equal(big[:512], big[-512:])


def test_resconv_spin_exchange_sweep_bit_exact(cuda):
    from quantax_gb300 import _lib as Lb
    L, B, Cc = 4, 2, 8
    net = Net(L, B, Cc, True, seed=2, bias_std=0.3)
    n = L * L
    nbr = lattice.neighbor_table((L, L), 1)
    s0 = metropolis.init_fixed_up(32, n, n // 2, 4)
    seed, nsteps = 77, 24
    want, want_lp, st = metropolis.sweep(lambda x: net.oracle.log_psi(x).real, s0, nsteps, seed, 0,
                                         proposal="exchange", nbr_table=nbr, hop=1)
    assert st["min_margin"] > 1e-4
    packed = _pack(s0)
    lp = torch.empty((32, 2), dtype=torch.float32, device="cuda")
    acc = torch.empty(32, dtype=torch.int32, device="cuda")
    nbr_t = torch.as_tensor(nbr).cuda()
    ws = torch.empty(Lb.lib().qgx_resconv_sweep_workspace_bytes(L, 32), dtype=torch.uint8, device="cuda")
    Lb.call("qgx_resconv_sweep", Lb.ptr(net.table), L, B, Cc, 1, 0, Lb.ptr(packed), Lb.ptr(lp), Lb.ptr(acc), 32, nsteps,
            seed, 0, 2.0, Lb.ptr(nbr_t), nbr.shape[1], 1, Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    assert (_unpack(packed, n) == want).all()
    assert (acc.cpu().numpy() == st["accepts"]).all()
    assert np.abs(lp.cpu().numpy()[:, 0] - want_lp).max() < 2e-4


@pytest.mark.parametrize("cplx", [True, False])
def test_resconv_local_energy_j1j2(cuda, cplx):
    import quantax_gb300.operator as O
    from quantax_gb300 import _lib as Lb
    L, B, Cc = 4, 2, 8
    net = Net(L, B, Cc, cplx, seed=5)
    n = L * L
    ops = oops.square_j1j2(L, 0.5, True)
    op = O.CompiledOperator(*O.compile_op_list(ops))
    s = metropolis.init_fixed_up(40, n, n // 2, 9)
    want = oops.local_energy(s, ops, net.oracle.log_psi)
    max_conn = len(op.host["f1"]) + len(op.host["f2"])
    ws = torch.empty(Lb.lib().qgx_resconv_eloc_workspace_bytes(L, 40, max_conn), dtype=torch.uint8, device="cuda")
    er = torch.empty(40, dtype=torch.float64, device="cuda")
    ei = torch.empty(40, dtype=torch.float64, device="cuda")
    Lb.call("qgx_resconv_eloc", Lb.ptr(net.table), L, B, Cc, int(cplx), 0, C.byref(op.struct), Lb.ptr(_pack(s)), 40,
            Lb.ptr(er), Lb.ptr(ei), Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    got = er.cpu().numpy() + 1j * ei.cpu().numpy()
    np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-4 * np.abs(want).max())


@pytest.mark.parametrize("L,B,Cc,cplx", [(4, 2, 8, True), (5, 3, 4, False), (10, 8, 16, True)])
def test_resconv_jacobian(cuda, L, B, Cc, cplx):
    from quantax_gb300 import _lib as Lb
    net = Net(L, B, Cc, cplx, seed=7)
    n = L * L
    ns = 6
    s = metropolis.init_fixed_up(ns, n, n // 2, 2)
    npar = net.p.size
    O = torch.full((2 * ns, npar), float("nan"), dtype=torch.float32, device="cuda")
    ws = torch.empty(Lb.lib().qgx_resconv_jacobian_workspace_bytes(L, B, Cc), dtype=torch.uint8, device="cuda")
    Lb.call("qgx_resconv_jacobian", Lb.ptr(net.table), L, B, Cc, int(cplx), Lb.ptr(_pack(s)), ns, Lb.ptr(O[:ns]),
            Lb.ptr(O[ns:]) if cplx else None, npar, Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    want = net.oracle.jacobian(s)
    got = O.cpu().numpy().astype(np.float64)
    scale = np.abs(want).max()
    np.testing.assert_allclose(got[:ns], want.real, rtol=2e-3, atol=2e-4 * scale)
    if cplx:
        np.testing.assert_allclose(got[ns:], want.imag, rtol=2e-3, atol=2e-4 * scale)


def test_resconv_sr_step_matches_oracle(cuda):
    """J1-J2 (J2 = 0.5, MSR) on 4x4, ResConv(2 blocks, 8 channels, complex output),
    SpinExchange, MinSR with a diagonal shift: one full step through the public API against
    the oracle on identical samples. Stated tolerance: 1e-2 relative 2-norm for the update
    (FP32 network values through a conditioned solve), 1e-5 relative for the energy."""
    import quantax_gb300 as qtx
    from oracle import sr as osr
    qtx.set_random_seed(3)
    qtx.set_default_dtype(np.complex128)
    try:
        qtx.sites.Square(4, Nparticles=(8, 8))
        H = qtx.operator.Heisenberg(J=[1.0, 0.5], n_neighbor=[1, 2], msr=True)
        model = qtx.model.ResConv(2, 8, out_dtype=np.complex64)
        state = qtx.state.Variational(model)
        sampler = qtx.sampler.SpinExchange(state, 128, thermal_steps=64, sweep_steps=32)
        opt = qtx.optimizer.SR(state, H, solver=qtx.optimizer.auto_shift_eig(ashift=1e-3))
        samples = sampler.sweep()
        step = opt.get_step(samples).cpu().numpy()
        s = samples.spins.cpu().numpy()
        onet = resconv.ResConv(state.params.cpu().numpy(), 4, 2, 8, True)
        ops = oops.square_j1j2(4, 0.5, True)
        E = oops.local_energy(s, ops, onet.log_psi)
        eb, em, var = osr.ebar(E)
        Ob = osr.obar(onet.jacobian(s))
        x = osr.solve(Ob, eb, lambda A, b: osr.auto(A, b, "shift", rshift=1e-6, ashift=1e-3), complex_out=True)
        assert abs(opt.energy - em) <= 1e-5 * abs(em)
        assert np.linalg.norm(step - x) / np.linalg.norm(x) < 1e-2
        state.update(torch.as_tensor(step).cuda() * 1e-2)
    finally:
        qtx.set_default_dtype(np.float64)


@pytest.mark.parametrize("prec", [0, 2])
def test_resconv_sweep_graph_replay_equals_one_sweep(cuda, prec):
    """A sweep is captured once into a CUDA graph and replayed; the Philox step base is read
    from the workspace, so two replays starting at steps 0 and 12 give exactly the 24-step
    sweep (configurations, log psi and the accepts of each part)."""
    from quantax_gb300 import _lib as Lb
    L, B, Cc, ns = 4, 2, 8, 48
    net = Net(L, B, Cc, True, seed=6, bias_std=0.3)
    nbr = torch.as_tensor(lattice.neighbor_table((L, L), 1)).cuda()
    s0 = _pack(metropolis.init_fixed_up(ns, 16, 8, 11))

    def sweep(packed, nsteps, step0, ws):
        lp = torch.empty((ns, 2), dtype=torch.float32, device="cuda")
        acc = torch.empty(ns, dtype=torch.int32, device="cuda")
        Lb.call("qgx_resconv_sweep", Lb.ptr(net.table), L, B, Cc, 1, prec, Lb.ptr(packed), Lb.ptr(lp), Lb.ptr(acc),
                ns, nsteps, 5, step0, 2.0, Lb.ptr(nbr), nbr.shape[1], 1, Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
        return lp, acc

    ws = torch.empty(Lb.lib().qgx_resconv_sweep_workspace_bytes(L, ns), dtype=torch.uint8, device="cuda")
    one = s0.clone()
    lp1, acc1 = sweep(one, 24, 0, ws)
    two = s0.clone()
    _, a = sweep(two, 12, 0, ws)
    lp2, b = sweep(two, 12, 12, ws)  # same buffers and sizes: the same graph, another step base
    assert torch.equal(one, two)
    assert torch.equal(lp1, lp2)
    assert torch.equal(acc1, a + b)
