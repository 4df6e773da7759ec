"""Symmetry projection of RBM_Dense on the GPU (qgx_rbm_*_symm) against the oracle's
projection of the FP64 RBM (oracle/rbm.py, oracle/symmetry.py); and the public
Variational(RBM_Dense, symm=...) path through one SR step.

The reference projects any model (quantax/state/variational.py:261-266,
quantax/symmetry/symmetry.py:325-392). Unlike the ResConv, an RBM is not translation invariant,
so translation groups with a momentum are meaningful projections here.

Stated tolerances, FP32 device against FP64 oracle:
- log psi of one image: 1e-4 absolute;
- sums over the group: a sum that cancels amplifies errors by
  kappa = sum_g |w_g psi_g| / |psi_symm|, so log psi_symm is held to 1e-4 x kappa per
  configuration;
- E_loc: 1e-3 of the largest |E_loc|;
- O: 2e-3 relative plus 2e-4 of the largest entry, times kappa."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import lattice, metropolis, operators as oops, rbm, symmetry as osym

from test_gpu_rbm import Rbm, pack, unpack

pytestmark = pytest.mark.gpu

L = 4
N = L * L


def _chain_translations(n):
    return np.stack([np.roll(np.arange(n), -k) for k in range(n)])


def _groups():
    rot, flip = osym.rotation90(L), osym.flip0(L)
    tx, ty = osym.translation(L, 1, 0), osym.translation(L, 0, 1)
    c4v = osym.product(osym.group([rot], [0]), osym.group([flip], [0]))
    return {
        "c4v_z2": (*c4v, 1),
        # complex characters: momentum (pi/2, 0), 16 translations
        "trans_k": (*osym.group([tx, ty], [1, 0]), 0),
        # real characters with signs: B1 of C4v, odd under spin inversion
        "b1_odd": (*osym.product(osym.group([rot], [2], False), osym.group([flip], [0], False)), -1),
        # translations x C4v x spin inversion: 256 elements
        "full": (*osym.product(osym.group([tx, ty], [0, 0]), c4v), 1),
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

    def kappa(self, log_psi_fn, s):
        ss = osym.symm_spins(s, self.perms, self.z2)
        ns, ng, n = ss.shape
        lg = log_psi_fn(ss.reshape(-1, n)).reshape(ns, ng)
        top = (np.abs(osym.weights(self.chars, self.z2))[None] * np.exp(lg)).sum(axis=1)
        with np.errstate(divide="ignore", over="ignore"):
            return top / np.exp(self.log_psi(log_psi_fn, s).real)

    def configs(self, log_psi_fn, ns, seed, n=N, fixed=True):
        """ns configurations whose projection does not vanish (kappa < 1e3)."""
        pool = metropolis.init_fixed_up(8 * ns, n, n // 2, seed) if fixed else metropolis.init_uniform(8 * ns, n, seed)
        keep = pool[self.kappa(log_psi_fn, pool) < 1e3]
        assert keep.shape[0] >= ns
        return keep[:ns]


def _net(n, m, seed, vb=False, std=0.25):
    W, b, a = rbm.init_normal(n, m, std, seed=seed, visible_bias=vb)
    return rbm.RBM(W, b, a), Rbm(W, b, a)


def _ws(nbytes):
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device="cuda")


def _log_psi_dev(dev, sym, s):
    from quantax_gb300 import _lib as Lb
    ns = s.shape[0]
    out = torch.empty((ns, 2), dtype=torch.float32, device="cuda")
    ws = _ws(Lb.lib().qgx_rbm_log_psi_symm_workspace_bytes(dev.N, ns, sym.nsymm))
    Lb.call("qgx_rbm_log_psi_symm", Lb.ptr(dev.table), dev.N, dev.M, C.byref(sym.struct), Lb.ptr(pack(s)), ns,
            Lb.ptr(out), Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    o = out.cpu().numpy().astype(np.float64)
    return o[:, 0] + 1j * o[:, 1]


def _phase_diff(a, b):
    return np.abs(np.angle(np.exp(1j * (a - b))))


@pytest.mark.parametrize("group", ["c4v_z2", "trans_k", "b1_odd", "full"])
@pytest.mark.parametrize("m,vb", [(32, False), (200, True)])
def test_rbm_symm_log_psi(cuda, group, m, vb):
    onet, dev = _net(N, m, seed=3 + m, vb=vb)
    sym = Symm(*_groups()[group])
    s = sym.configs(onet.log_psi, 48, 5)
    want = sym.log_psi(onet.log_psi, s)
    got = _log_psi_dev(dev, sym, s)
    kappa = sym.kappa(onet.log_psi, s)
    assert (np.abs(got.real - want.real) <= 1e-4 * kappa).all()
    assert (_phase_diff(got.imag, want.imag) <= 1e-4 * kappa).all()


@pytest.mark.parametrize("group", ["c4v_z2", "trans_k", "b1_odd"])
def test_rbm_symm_local_energy(cuda, group):
    """E_loc of the projected RBM for J1-J2 (J2 = 0.5, MSR) on the 4 x 4 square."""
    import quantax_gb300.operator as O
    from quantax_gb300 import _lib as Lb
    onet, dev = _net(N, 32, seed=11)
    sym = Symm(*_groups()[group])
    ops = oops.square_j1j2(L, 0.5, True)
    op = O.CompiledOperator(*O.compile_op_list(ops))
    ns = 40
    s = sym.configs(onet.log_psi, ns, 9)
    want = oops.local_energy(s, ops, lambda x: sym.log_psi(onet.log_psi, x))
    max_conn = len(op.host["f1"]) + len(op.host["f2"])
    ws = _ws(Lb.lib().qgx_rbm_eloc_symm_workspace_bytes(N, ns, max_conn, sym.nsymm))
    er = torch.empty(ns, dtype=torch.float64, device="cuda")
    ei = torch.empty(ns, dtype=torch.float64, device="cuda")
    Lb.call("qgx_rbm_eloc_symm", Lb.ptr(dev.table), N, dev.M, C.byref(sym.struct), C.byref(op.struct),
            Lb.ptr(pack(s)), ns, Lb.ptr(er), Lb.ptr(ei), Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    got = er.cpu().numpy() + 1j * ei.cpu().numpy()
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-3 * np.abs(want).max())


@pytest.mark.parametrize("group,vb", [("c4v_z2", False), ("trans_k", True), ("b1_odd", False)])
def test_rbm_symm_jacobian(cuda, group, vb):
    """d log psi_symm / d params against the oracle's weighted sum of the images' closed forms."""
    from quantax_gb300 import _lib as Lb
    onet, dev = _net(N, 32, seed=7, vb=vb)
    sym = Symm(*_groups()[group])
    ns = 6
    s = sym.configs(onet.log_psi, ns, 2)
    npar = onet.nparams
    O = torch.full((2 * ns, npar), float("nan"), dtype=torch.float32, device="cuda")
    ws = _ws(Lb.lib().qgx_rbm_jacobian_symm_workspace_bytes(N, dev.M, int(vb), ns, sym.nsymm))
    Lb.call("qgx_rbm_jacobian_symm", Lb.ptr(dev.table), N, dev.M, int(vb), C.byref(sym.struct), Lb.ptr(pack(s)), ns,
            Lb.ptr(O[:ns]), Lb.ptr(O[ns:]), npar, Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    want = osym.jacobian_symm(onet.log_psi, onet.jacobian, s, sym.perms, sym.chars, sym.z2)
    kappa = sym.kappa(onet.log_psi, s)[:, None]
    got = O.cpu().numpy().astype(np.float64)
    bound = (2e-3 * np.abs(want) + 2e-4 * np.abs(want).max()) * kappa
    assert (np.abs(got[:ns] - want.real) <= bound).all()
    assert (np.abs(got[ns:] - want.imag) <= bound).all()


def test_rbm_symm_jacobian_chunks(cuda):
    """More samples than one pass of image rows holds (2^26 floats): the chunked passes give the
    same rows as one sample at a time."""
    from quantax_gb300 import _lib as Lb
    onet, dev = _net(N, 200, seed=13, vb=True)
    sym = Symm(*_groups()["full"])  # 256 images x 3416 parameters: 76 samples per pass
    npar = onet.nparams
    ns = 160
    s = metropolis.init_fixed_up(ns, N, N // 2, 21)

    def run(x):
        k = x.shape[0]
        O = torch.empty((k, npar), dtype=torch.float32, device="cuda")
        ws = _ws(Lb.lib().qgx_rbm_jacobian_symm_workspace_bytes(N, dev.M, 1, k, sym.nsymm))
        Lb.call("qgx_rbm_jacobian_symm", Lb.ptr(dev.table), N, dev.M, 1, C.byref(sym.struct), Lb.ptr(pack(x)), k,
                Lb.ptr(O), None, npar, Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
        return O

    whole = run(s)
    for i in (0, 75, 76, 159):
        assert torch.equal(whole[i], run(s[i:i + 1])[0]), i


@pytest.mark.parametrize("proposal", ["exchange", "flip"])
def test_rbm_symm_sweep_bit_exact(cuda, proposal):
    """Metropolis sweep of the projected RBM: the same chains, accepts and log psi as the oracle's
    Metropolis on the projected log psi (decisions at least 1e-4 from the threshold).
    SpinExchange on the 4 x 4 square with C4v x Z2; LocalFlip on a 12-site chain projected on
    zero momentum (no Sz constraint)."""
    from quantax_gb300 import _lib as Lb
    if proposal == "exchange":
        n, m, seed, nsteps = N, 32, 77, 24
        perms, chars, z2 = _groups()["c4v_z2"]
        nbr = lattice.neighbor_table((L, L), 1)
        s0 = metropolis.init_fixed_up(32, n, n // 2, 4)
        kw = dict(proposal="exchange", nbr_table=nbr, hop=1)
        prop, nbr_t, z = Lb.PROPOSAL_SPIN_EXCHANGE, torch.as_tensor(nbr).cuda(), nbr.shape[1]
    else:
        n, m, seed, nsteps = 12, 24, 31, 30
        perms, chars, z2 = _chain_translations(n), np.ones(n, dtype=np.complex128), 0
        s0 = metropolis.init_uniform(32, n, 6)
        kw = dict(proposal="flip")
        prop, nbr_t, z = Lb.PROPOSAL_LOCAL_FLIP, None, 0
    onet, dev = _net(n, m, seed=2, std=0.3)
    sym = Symm(perms, chars, z2)
    ns = s0.shape[0]
    want, want_lp, st = metropolis.sweep(lambda x: sym.log_psi(onet.log_psi, x).real, s0, nsteps, seed, 0, **kw)
    assert st["min_margin"] > 1e-4
    packed = pack(s0)
    lp = torch.empty((ns, 2), dtype=torch.float32, device="cuda")
    acc = torch.empty(ns, dtype=torch.int32, device="cuda")
    ws = _ws(Lb.lib().qgx_rbm_sweep_symm_workspace_bytes(n, ns, sym.nsymm))
    Lb.call("qgx_rbm_sweep_symm", Lb.ptr(dev.table), n, m, C.byref(sym.struct), Lb.ptr(packed), Lb.ptr(lp),
            Lb.ptr(acc), ns, nsteps, seed, 0, 2.0, prop, Lb.ptr(nbr_t), z, 1, Lb.ptr(ws), ws.numel(), Lb.stream_ptr())
    assert (unpack(packed, n) == want).all()
    assert (acc.cpu().numpy() == st["accepts"]).all()
    assert np.abs(lp.cpu().numpy()[:, 0] - want_lp).max() < 1e-4


def test_rbm_symm_state_sr_step(cuda):
    """Variational(RBM_Dense(32), symm=Rotation(pi/2) @ Flip() @ SpinInverse()) through the public
    API on the 4 x 4 J1-J2 model: sampler, energy and one MinSR update against the oracle on the
    same samples (stated: log psi 1e-3, energy 1e-5 relative, update 1e-2 relative 2-norm)."""
    import quantax_gb300 as qtx
    from oracle import sr as osr
    from quantax_gb300.symmetry import Flip, Rotation, SpinInverse
    qtx.set_random_seed(5)
    qtx.sites.Square(4, Nparticles=(8, 8))
    H = qtx.operator.Heisenberg(J=[1.0, 0.5], n_neighbor=[1, 2], msr=True)
    symm = Rotation(np.pi / 2) @ Flip() @ SpinInverse()
    model = qtx.model.RBM_Dense(32, init_std=0.1, seed=3)
    state = qtx.state.Variational(model, symm=symm)
    sampler = qtx.sampler.SpinExchange(state, 128, thermal_steps=64, sweep_steps=32)
    opt = qtx.optimizer.SR(state, H, solver=qtx.optimizer.auto_shift_eig(ashift=1e-3))
    samples = sampler.sweep()
    step = opt.get_step(samples).cpu().numpy()
    s = samples.spins.cpu().numpy()
    p = state.params.cpu().numpy().astype(np.float64)
    onet = rbm.RBM(p[:32 * 16].reshape(32, 16), p[32 * 16:32 * 16 + 32])
    perms, chars, z2 = _groups()["c4v_z2"]
    lpf = lambda x: osym.log_psi_symm(onet.log_psi, x, perms, chars, z2)
    lp_dev = samples.log_psi.cpu().numpy()
    assert np.abs(lp_dev.real - lpf(s).real).max() < 1e-3
    E = oops.local_energy(s, oops.square_j1j2(4, 0.5, True), lpf)
    eb, em, _ = osr.ebar(E.real)
    Ob = osr.obar(osym.jacobian_symm(onet.log_psi, onet.jacobian, s, perms, chars, z2).real)
    x = osr.solve(Ob, eb, lambda A, b: osr.auto(A, b, "shift", rshift=1e-6, ashift=1e-3), complex_out=False)
    assert abs(opt.energy - em) <= 1e-5 * abs(em)
    assert np.linalg.norm(step - x) / np.linalg.norm(x) < 1e-2


def test_rbm_symm_complex_characters_give_complex_rows(cuda):
    """With complex characters and a complex computation dtype the projected RBM is a
    real-to-complex state: its O rows are [Re; Im] and match the oracle."""
    import quantax_gb300 as qtx
    from quantax_gb300.symmetry import TransND
    qtx.set_random_seed(9)
    qtx.set_default_dtype(np.complex128)
    try:
        qtx.sites.Square(4, Nparticles=(8, 8))
        symm = TransND(sector=(1, 0))
        state = qtx.state.Variational(qtx.model.RBM_Dense(32, init_std=0.2, seed=4), symm=symm)
        assert state.is_complex and state.vs_type == qtx.state.VS_TYPE.real_to_complex
        s = metropolis.init_fixed_up(8, N, N // 2, 3)
        O = state.jacobian(s).cpu().numpy()
        p = state.params.cpu().numpy().astype(np.float64)
        onet = rbm.RBM(p[:32 * 16].reshape(32, 16), p[32 * 16:32 * 16 + 32])
        perms = symm.perm
        chars = symm.character
        want = osym.jacobian_symm(onet.log_psi, onet.jacobian, s, perms, chars, 0)
        bound = 2e-3 * np.abs(want) + 2e-4 * np.abs(want).max()
        kappa = Symm(perms, chars, 0).kappa(onet.log_psi, s)[:, None]
        assert (np.abs(O - want) <= bound * kappa).all()
    finally:
        qtx.set_default_dtype(np.float64)
