"""Symmetry projection on the GPU (qgx_resconv_*_symm) against the oracle's projection of the
FP64 ResConv (oracle/symmetry.py), with the oracle's own group tables; and the public
Variational(symm=...) path through one SR step.

Stated tolerances: the per-element values carry the unsymmetrised bounds (log psi 2e-4 FP32,
5e-3 TF32, 4e-2 BF16); a sum over the group that cancels amplifies them by
kappa = sum_g |w_g psi_g| / |psi_symm|, so log psi_symm is held to bound x kappa per
configuration."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import lattice, metropolis, operators as oops, resconv, symmetry as osym

from test_gpu_resconv import Net, _pack, _unpack

pytestmark = pytest.mark.gpu

L = 4
N = L * L


def _groups():
    rot, flip = osym.rotation90(L), osym.flip0(L)
    return {
        # Rotation(pi/2) @ Flip() @ SpinInverse(): the J1-J2 notebook's projection
        "c4v_z2": (*osym.product(osym.group([rot], [0]), osym.group([flip], [0])), 1),
        # complex characters: sector 1 of the rotations (powers of -i). Translations with a
        # momentum would not do: the network is translation invariant already (periodic
        # convolutions and a mean over sites), so every non-zero momentum projects it to 0
        "rot_c": (*osym.group([rot], [1]), 0),
        # real characters with signs: B1 of C4v, odd under spin inversion
        "b1_odd": (*osym.product(osym.group([rot], [2], False), osym.group([flip], [0], False)), -1),
    }


class Symm:
    def __init__(self, perms, chars, z2):
        from quantax_gb300 import _lib as Lb
        self.perms, self.chars, self.z2 = perms, chars, z2
        w = osym.weights(chars, z2)
        self.perm_t = torch.as_tensor(perms.astype(np.int16)).cuda().contiguous()
        self.w_t = torch.as_tensor(np.stack([w.real, w.imag], 1).reshape(-1)).cuda().contiguous()
        self.struct = Lb.Symm(C.c_void_p(self.perm_t.data_ptr()), C.c_void_p(self.w_t.data_ptr()), perms.shape[0], z2)
        self.nsymm = perms.shape[0] * (2 if z2 else 1)

    def log_psi(self, log_psi_fn, s):
        return osym.log_psi_symm(log_psi_fn, s, self.perms, self.chars, self.z2)

    def top(self, log_psi_fn, s):
        """sum_g |w_g psi(T_g s)|"""
        ss = osym.symm_spins(s, self.perms, self.z2)
        ns, ng, n = ss.shape
        lg = log_psi_fn(ss.reshape(-1, n)).reshape(ns, ng)
        return (np.abs(osym.weights(self.chars, self.z2))[None] * np.exp(lg.real)).sum(axis=1)

    def kappa(self, log_psi_fn, s):
        with np.errstate(divide="ignore", over="ignore"):
            return self.top(log_psi_fn, s) / np.exp(self.log_psi(log_psi_fn, s).real)

    def configs(self, log_psi_fn, ns, seed):
        """ns configurations whose projection does not vanish (kappa < 1e3): the ones a
        Metropolis chain visits."""
        pool = metropolis.init_fixed_up(8 * ns, N, N // 2, seed)
        keep = pool[self.kappa(log_psi_fn, pool) < 1e3]
        assert keep.shape[0] >= ns
        return keep[:ns]


def _log_psi_symm_dev(net, sym, s, prec):
    from quantax_gb300 import _lib as Lb
    ns = s.shape[0]
    out = torch.empty((ns, 2), dtype=torch.float32, device="cuda")
    packed = _pack(s)
    ws = torch.empty(Lb.lib().qgx_resconv_log_psi_symm_workspace_bytes(L, ns, sym.nsymm), dtype=torch.uint8,
                     device="cuda")
    Lb.call("qgx_resconv_log_psi_symm", Lb.ptr(net.table), L, net.B, net.C, int(net.cplx), prec, C.byref(sym.struct),
            Lb.ptr(packed), ns, Lb.ptr(out), Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    o = out.cpu().numpy().astype(np.float64)
    return o[:, 0] + 1j * o[:, 1]


@pytest.mark.parametrize("group,cplx", [("c4v_z2", True), ("rot_c", True), ("b1_odd", False), ("c4v_z2", False)])
@pytest.mark.parametrize("prec,tol", [(0, 2e-4), (1, 5e-3), (2, 4e-2)])
def test_symm_log_psi(cuda, group, cplx, prec, tol):
    net = Net(L, 2, 8, cplx, seed=3, bias_std=0.2)
    sym = Symm(*_groups()[group])
    s = metropolis.init_fixed_up(48, N, N // 2, 5)
    got = _log_psi_symm_dev(net, sym, s, prec)
    want = sym.log_psi(net.oracle.log_psi, s)
    kappa = sym.kappa(net.oracle.log_psi, s)
    # configurations the representation forces to zero: the device sum is rounding only
    zero = ~(kappa < 1e8)
    top = sym.top(net.oracle.log_psi, s)
    assert (np.exp(got.real[zero]) <= 2 * tol * top[zero]).all()
    live = ~zero
    assert live.sum() >= 16
    err_re = np.abs(got.real[live] - want.real[live])
    err_ph = np.abs(np.angle(np.exp(1j * (got.imag[live] - want.imag[live]))))
    assert (err_re <= tol * kappa[live]).all(), (err_re / kappa[live]).max()
    assert (err_ph <= tol * kappa[live]).all(), (err_ph / kappa[live]).max()
    if not cplx and group == "b1_odd":
        # a real projected state is negative on part of the configurations: phase pi
        ph = np.abs(np.angle(np.exp(1j * want.imag[live])))
        assert ((ph < 1e-6) | (ph > np.pi - 1e-6)).all() and (ph > 1).any()


@pytest.mark.parametrize("group,cplx", [("c4v_z2", True), ("rot_c", True), ("b1_odd", False)])
def test_symm_local_energy(cuda, group, cplx):
    """E_loc of the projected state, J1-J2 (J2 = 0.5, MSR): stated 1e-3 of max |E_loc|."""
    import quantax_gb300.operator as O
    from quantax_gb300 import _lib as Lb
    net = Net(L, 2, 8, cplx, seed=5, bias_std=0.2)
    sym = Symm(*_groups()[group])
    ops = oops.square_j1j2(L, 0.5, True)
    op = O.CompiledOperator(*O.compile_op_list(ops))
    ns = 40
    s = sym.configs(net.oracle.log_psi, ns, 9)
    want = oops.local_energy(s, ops, lambda x: sym.log_psi(net.oracle.log_psi, x))
    max_conn = len(op.host["f1"]) + len(op.host["f2"])
    ws = torch.empty(Lb.lib().qgx_resconv_eloc_symm_workspace_bytes(L, ns, max_conn, sym.nsymm), dtype=torch.uint8,
                     device="cuda")
    er = torch.empty(ns, dtype=torch.float64, device="cuda")
    ei = torch.empty(ns, dtype=torch.float64, device="cuda")
    packed = _pack(s)
    Lb.call("qgx_resconv_eloc_symm", Lb.ptr(net.table), L, 2, 8, int(cplx), 0, C.byref(sym.struct), C.byref(op.struct),
            Lb.ptr(packed), ns, Lb.ptr(er), Lb.ptr(ei), Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    got = er.cpu().numpy() + 1j * ei.cpu().numpy()
    if not cplx:
        want = want.real
        got = got.real
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-3 * np.abs(want).max())


@pytest.mark.parametrize("group,cplx", [("c4v_z2", True), ("rot_c", True), ("b1_odd", False)])
def test_symm_jacobian(cuda, group, cplx):
    """d log psi_symm / d params against the oracle's weighted sum over the group: stated
    2e-3 relative plus 2e-4 of the largest entry, times kappa."""
    from quantax_gb300 import _lib as Lb
    net = Net(L, 2, 8, cplx, seed=7, bias_std=0.2)
    sym = Symm(*_groups()[group])
    ns = 6
    s = sym.configs(net.oracle.log_psi, ns, 2)
    npar = net.p.size
    O = torch.full((2 * ns, npar), float("nan"), dtype=torch.float32, device="cuda")
    ws = torch.empty(Lb.lib().qgx_resconv_jacobian_symm_workspace_bytes(L, 2, 8, ns, sym.nsymm), dtype=torch.uint8,
                     device="cuda")
    packed = _pack(s)
    Lb.call("qgx_resconv_jacobian_symm", Lb.ptr(net.table), L, 2, 8, int(cplx), C.byref(sym.struct), Lb.ptr(packed),
            ns, Lb.ptr(O[:ns]), Lb.ptr(O[ns:]) if cplx else None, npar, Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    want = osym.jacobian_symm(net.oracle.log_psi, net.oracle.jacobian, s, sym.perms, sym.chars, sym.z2)
    kappa = sym.kappa(net.oracle.log_psi, s)[:, None]
    got = O.cpu().numpy().astype(np.float64)
    scale = np.abs(want).max()
    bound = (2e-3 * np.abs(want) + 2e-4 * scale) * kappa
    assert (np.abs(got[:ns] - want.real) <= bound).all()
    if cplx:
        assert (np.abs(got[ns:] - want.imag) <= bound).all()


def test_symm_sweep_bit_exact(cuda):
    """SpinExchange sweep of the projected state: the same chains, accepts and log psi as the
    oracle's Metropolis on the projected log psi (decisions at least 1e-4 from the threshold)."""
    from quantax_gb300 import _lib as Lb
    net = Net(L, 2, 8, True, seed=2, bias_std=0.3)
    sym = Symm(*_groups()["c4v_z2"])
    nbr = lattice.neighbor_table((L, L), 1)
    ns, seed, nsteps = 32, 77, 24
    s0 = metropolis.init_fixed_up(ns, N, N // 2, 4)
    want, want_lp, st = metropolis.sweep(lambda x: sym.log_psi(net.oracle.log_psi, x).real, s0, nsteps, seed, 0,
                                         proposal="exchange", nbr_table=nbr, hop=1)
    assert st["min_margin"] > 1e-4
    packed = _pack(s0)
    lp = torch.empty((ns, 2), dtype=torch.float32, device="cuda")
    acc = torch.empty(ns, dtype=torch.int32, device="cuda")
    nbr_t = torch.as_tensor(nbr).cuda()
    ws = torch.empty(Lb.lib().qgx_resconv_sweep_symm_workspace_bytes(L, ns, sym.nsymm), dtype=torch.uint8,
                     device="cuda")
    Lb.call("qgx_resconv_sweep_symm", Lb.ptr(net.table), L, 2, 8, 1, 0, C.byref(sym.struct), Lb.ptr(packed),
            Lb.ptr(lp), Lb.ptr(acc), ns, nsteps, seed, 0, 2.0, Lb.ptr(nbr_t), nbr.shape[1], 1, Lb.ptr(ws), ws.numel(),
            Lb.stream_ptr())
    assert (_unpack(packed, N) == want).all()
    assert (acc.cpu().numpy() == st["accepts"]).all()
    assert np.abs(lp.cpu().numpy()[:, 0] - want_lp).max() < 2e-4


def test_symm_state_sr_step(cuda):
    """The J1-J2 notebook's projected state, Variational(model, symm=Rotation(pi/2) @ Flip() @
    SpinInverse()), through the public API: sampler, energy and one MinSR update against the
    oracle on the same samples (stated: energy 1e-5 relative, update 1e-2 relative 2-norm)."""
    import quantax_gb300 as qtx
    from oracle import sr as osr
    from quantax_gb300.symmetry import Flip, Rotation, SpinInverse
    qtx.set_random_seed(3)
    qtx.set_default_dtype(np.complex128)
    try:
        qtx.sites.Square(4, Nparticles=(8, 8))
        H = qtx.operator.Heisenberg(J=[1.0, 0.5], n_neighbor=[1, 2], msr=True)
        symm = Rotation(np.pi / 2) @ Flip() @ SpinInverse()
        assert symm.nsymm == 16
        state = qtx.state.Variational(qtx.model.ResConv(2, 8, out_dtype=np.complex64), symm=symm)
        sampler = qtx.sampler.SpinExchange(state, 128, thermal_steps=64, sweep_steps=32)
        opt = qtx.optimizer.SR(state, H, solver=qtx.optimizer.auto_shift_eig(ashift=1e-3))
        samples = sampler.sweep()
        step = opt.get_step(samples).cpu().numpy()
        s = samples.spins.cpu().numpy()
        onet = resconv.ResConv(state.params.cpu().numpy(), 4, 2, 8, True)
        perms, chars, z2 = _groups()["c4v_z2"]
        lpf = lambda x: osym.log_psi_symm(onet.log_psi, x, perms, chars, z2)
        lp_dev = samples.log_psi.cpu().numpy()
        assert np.abs(lp_dev.real - lpf(s).real).max() < 2e-4 * 10
        E = oops.local_energy(s, oops.square_j1j2(4, 0.5, True), lpf)
        eb, em, _ = osr.ebar(E)
        Ob = osr.obar(osym.jacobian_symm(onet.log_psi, onet.jacobian, s, perms, chars, z2))
        x = osr.solve(Ob, eb, lambda A, b: osr.auto(A, b, "shift", rshift=1e-6, ashift=1e-3), complex_out=True)
        assert abs(opt.energy - em) <= 1e-5 * abs(em)
        assert np.linalg.norm(step - x) / np.linalg.norm(x) < 1e-2
    finally:
        qtx.set_default_dtype(np.float64)
