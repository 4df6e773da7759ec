"""GPU parity of the RBM kernels against the oracle, through the qgx C ABI."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import lattice, metropolis, operators as oops, philox, rbm

pytestmark = pytest.mark.gpu


def lib():
    from quantax_gb300 import _lib
    return _lib


def pack(s):
    s = np.asarray(s)
    ns, n = s.shape
    nw = (n + 31) // 32
    out = np.zeros((ns, nw), dtype=np.uint32)
    for j in range(n):
        out[:, j // 32] |= (s[:, j] > 0).astype(np.uint32) << np.uint32(j % 32)
    return torch.as_tensor(out.view(np.int32)).cuda()


def unpack(t, n):
    w = t.cpu().numpy().view(np.uint32)
    out = np.empty((w.shape[0], n), dtype=np.int8)
    for j in range(n):
        out[:, j] = ((w[:, j // 32] >> np.uint32(j % 32)) & 1).astype(np.int8) * 2 - 1
    return out


class Rbm:
    """Device table of an explicit RBM, prepared through qgx_rbm_prepare."""

    def __init__(self, W, b, a=None):
        L = lib()
        self.M, self.N = W.shape
        self.W = torch.as_tensor(W, dtype=torch.float32).cuda()
        self.b = torch.as_tensor(b, dtype=torch.float32).cuda()
        self.a = None if a is None else torch.as_tensor(a, dtype=torch.float32).cuda()
        nf = L.lib().qgx_rbm_table_floats(self.N, self.M)
        self.table = torch.empty(nf, dtype=torch.float32, device="cuda")
        L.call("qgx_rbm_prepare", L.ptr(self.W), L.ptr(self.b), L.ptr(self.a), self.N, self.M, L.ptr(self.table),
               L.stream_ptr())

    def log_psi(self, packed):
        L = lib()
        out = torch.empty(packed.shape[0], dtype=torch.float32, device="cuda")
        L.call("qgx_rbm_log_psi", L.ptr(self.table), self.N, self.M, L.ptr(packed), packed.shape[0], L.ptr(out),
               L.stream_ptr())
        return out

    def sweep(self, packed, nsteps, seed, step0=0, reweight=2.0, proposal=0, nbr=None, z=0, hop=1):
        L = lib()
        ns = packed.shape[0]
        lp = torch.empty(ns, dtype=torch.float32, device="cuda")
        acc = torch.empty(ns, dtype=torch.int32, device="cuda")
        L.call("qgx_rbm_sweep", L.ptr(self.table), self.N, self.M, L.ptr(packed), L.ptr(lp), L.ptr(acc), ns, nsteps,
               seed, step0, reweight, proposal, L.ptr(nbr), z, hop, L.stream_ptr())
        return lp, acc


def compiled(op_list):
    import quantax_gb300.operator as O
    return O.CompiledOperator(*O.compile_op_list(op_list))


def test_philox_device_matches_known_answers(cuda):
    L = lib()
    ctr = np.array([[0, 0, 0, 0], [0xFFFFFFFF] * 4, [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344]], np.uint32)
    keys = [[0, 0], [0xFFFFFFFF] * 2, [0xA4093822, 0x299F31D0]]
    for c, k in zip(ctr, keys):
        ct = torch.as_tensor(c.view(np.int32)).cuda()
        kt = torch.as_tensor(np.array(k, np.uint32).view(np.int32)).cuda()
        out = torch.empty(4, dtype=torch.int32, device="cuda")
        L.call("qgx_philox4x32_10", L.ptr(ct), L.ptr(kt), L.ptr(out), 1, L.stream_ptr())
        assert out.cpu().numpy().view(np.uint32).tolist() == philox.philox4x32_10(c, k).tolist()


def test_init_configurations_bit_exact(cuda):
    L = lib()
    for ns, n, seed in [(64, 8, 3), (100, 70, 11), (37, 100, 5)]:
        packed = torch.empty((ns, (n + 31) // 32), dtype=torch.int32, device="cuda")
        L.call("qgx_spins_init_uniform", L.ptr(packed), ns, n, seed, L.stream_ptr())
        assert (unpack(packed, n) == metropolis.init_uniform(ns, n, seed)).all()
        w = packed.cpu().numpy().view(np.uint32)
        if n % 32:
            assert (w[:, -1] >> np.uint32(n % 32) == 0).all()  # bits beyond n stay clear
    for ns, n, nup, seed in [(50, 16, 8, 6), (40, 100, 50, 9), (10, 33, 7, 1)]:
        packed = torch.empty((ns, (n + 31) // 32), dtype=torch.int32, device="cuda")
        L.call("qgx_spins_init_fixed_up", L.ptr(packed), ns, n, nup, seed, L.stream_ptr())
        assert (unpack(packed, n) == metropolis.init_fixed_up(ns, n, nup, seed)).all()


def test_pack_unpack_round_trip(cuda):
    L = lib()
    s = metropolis.init_uniform(33, 77, 2)
    st = torch.as_tensor(s).cuda()
    packed = torch.empty((33, 3), dtype=torch.int32, device="cuda")
    L.call("qgx_spins_pack", L.ptr(st), L.ptr(packed), 33, 77, L.stream_ptr())
    assert (unpack(packed, 77) == s).all()
    back = torch.empty_like(st)
    L.call("qgx_spins_unpack", L.ptr(packed), L.ptr(back), 33, 77, L.stream_ptr())
    assert (back.cpu().numpy() == s).all()


@pytest.mark.parametrize("N,M,vb", [(8, 16, True), (64, 256, False), (100, 200, True), (30, 512, False)])
def test_log_psi(cuda, N, M, vb):
    W, b, a = rbm.init_normal(N, M, 0.1, seed=N + M, visible_bias=vb)
    dev = Rbm(W, b, a)
    net = rbm.RBM(W, b, a)
    s = metropolis.init_uniform(300, N, 4)
    got = dev.log_psi(pack(s)).cpu().numpy()
    np.testing.assert_allclose(got, net.log_psi(s), rtol=2e-6, atol=2e-5)


@pytest.mark.parametrize("N,M,std,ns,nsteps,vb", [(8, 16, 0.1, 64, 176, True), (64, 256, 0.05, 96, 128, False),
                                                   (20, 40, 0.3, 64, 100, True)])
def test_local_flip_sweep_bit_exact(cuda, N, M, std, ns, nsteps, vb):
    W, b, a = rbm.init_normal(N, M, std, seed=7, visible_bias=vb)
    net = rbm.RBM(W, b, a)
    s0 = metropolis.init_uniform(ns, N, 1)
    seed, step0 = 0x1234ABCD5678, 40
    want, want_lp, stats = metropolis.sweep(net.log_psi, s0, nsteps, seed, step0)
    # FP32 device decisions match the FP64 oracle when no accept test is a near tie
    assert stats["min_margin"] > 1e-5, "seeded case has a near-tie; pick another seed"
    dev = Rbm(W, b, a)
    packed = pack(s0)
    lp, acc = dev.sweep(packed, nsteps, seed, step0)
    assert (unpack(packed, N) == want).all()
    assert (acc.cpu().numpy() == stats["accepts"]).all()
    np.testing.assert_allclose(lp.cpu().numpy(), want_lp, rtol=2e-6, atol=2e-5)


def test_sweep_in_two_launches_equals_one(cuda):
    W, b, a = rbm.init_normal(16, 64, 0.2, seed=3, visible_bias=True)
    dev = Rbm(W, b, a)
    s0 = pack(metropolis.init_uniform(200, 16, 8))
    p1 = s0.clone()
    dev.sweep(p1, 50, 77, 0)
    p2 = s0.clone()
    dev.sweep(p2, 20, 77, 0)
    dev.sweep(p2, 30, 77, 20)
    assert torch.equal(p1, p2)


@pytest.mark.parametrize("shells", [1, [1, 2]])
def test_spin_exchange_sweep_bit_exact(cuda, shells):
    """SpinExchange with nearest neighbours, and with the first two shells
    (SpinExchange(state, n, n_neighbor=[1, 2]) of tutorials/neural_jastrow.ipynb): the
    neighbour rows are padded to the longest, the draws are the same."""
    L = 4
    N = L * L
    W, b, a = rbm.init_normal(N, 32, 0.2, seed=4, visible_bias=True)
    net = rbm.RBM(W, b, a)
    nbr = lattice.neighbor_table((L, L), shells)
    if shells != 1:
        assert nbr.shape[1] == 8
    s0 = metropolis.init_fixed_up(64, N, N // 2, 3)
    want, want_lp, stats = metropolis.sweep(net.log_psi, s0, 80, 99, 0, proposal="exchange", nbr_table=nbr, hop=1)
    assert stats["min_margin"] > 1e-5
    dev = Rbm(W, b, a)
    packed = pack(s0)
    nbr_t = torch.as_tensor(nbr).cuda()
    lp, acc = dev.sweep(packed, 80, 99, 0, proposal=1, nbr=nbr_t, z=nbr.shape[1], hop=1)
    got = unpack(packed, N)
    assert (got == want).all()
    assert (got.sum(axis=1) == 0).all()
    np.testing.assert_allclose(lp.cpu().numpy(), want_lp, rtol=2e-6, atol=2e-5)


@pytest.mark.parametrize("case", ["tfim8", "tfim64", "j1j2_4x4", "heis_chain"])
def test_local_energy(cuda, case):
    L = lib()
    if case.startswith("tfim"):
        N = int(case[4:])
        ops = oops.chain_tfim(N, h=0.8, J=1.1)
        s = metropolis.init_uniform(200, N, 5)
        M = 2 * N
    elif case == "j1j2_4x4":
        N = 16
        ops = oops.square_j1j2(4, 0.5, True)
        s = metropolis.init_fixed_up(200, N, 8, 5)
        M = 32
    else:
        N = 12
        ops = oops.heisenberg_op_list([lattice.neighbors((12,), 1)], [1.0], [1], False)
        s = metropolis.init_fixed_up(100, N, 6, 2)
        M = 24
    W, b, a = rbm.init_normal(N, M, 0.15, seed=1, visible_bias=True)
    net = rbm.RBM(W, b, a)
    want = oops.local_energy(s, ops, net.log_psi).real
    dev = Rbm(W, b, a)
    op = compiled(ops)
    out = torch.empty(s.shape[0], dtype=torch.float64, device="cuda")
    packed = pack(s)
    L.call("qgx_rbm_eloc", L.ptr(dev.table), N, M, C.byref(op.struct), L.ptr(packed), s.shape[0], L.ptr(out),
           L.stream_ptr())
    np.testing.assert_allclose(out.cpu().numpy(), want, rtol=1e-5, atol=1e-5 * np.abs(want).max())
    diag = torch.empty_like(out)
    L.call("qgx_operator_diag", C.byref(op.struct), L.ptr(packed), s.shape[0], N, L.ptr(diag), L.stream_ptr())
    want_diag = np.array([oops.connected(x, ops)[0] for x in s])
    np.testing.assert_allclose(diag.cpu().numpy(), want_diag, atol=1e-12)


@pytest.mark.parametrize("N,M,vb", [(8, 16, True), (64, 256, False), (10, 130, True), (7, 20, False)])
def test_jacobian_and_obar(cuda, N, M, vb):
    L = lib()
    W, b, a = rbm.init_normal(N, M, 0.2, seed=2, visible_bias=vb)
    net = rbm.RBM(W, b, a)
    ns = 300
    s = metropolis.init_uniform(ns, N, 6)
    dev = Rbm(W, b, a)
    packed = pack(s)
    npar = net.nparams
    O = torch.empty((ns, npar), dtype=torch.float32, device="cuda")
    L.call("qgx_rbm_jacobian", L.ptr(dev.table), N, M, int(vb), L.ptr(packed), ns, L.ptr(O), npar, L.stream_ptr())
    Oref = net.jacobian(s)
    np.testing.assert_allclose(O.cpu().numpy(), Oref, rtol=1e-5, atol=1e-6)
    r = np.random.default_rng(1).uniform(0.5, 1.5, ns)
    r = r / r.mean()
    rt = torch.as_tensor(r).cuda()
    ws = torch.empty(L.lib().qgx_rbm_obar_workspace_bytes(N, M, ns), dtype=torch.uint8, device="cuda")
    Ob = torch.empty((ns, npar), dtype=torch.float32, device="cuda")
    om = torch.empty(npar, dtype=torch.float64, device="cuda")
    L.call("qgx_rbm_obar", L.ptr(dev.table), N, M, int(vb), L.ptr(packed), L.ptr(rt), ns, L.ptr(Ob), npar, L.ptr(om),
           L.ptr(ws), ws.numel(), L.stream_ptr())
    from oracle import sr as osr
    np.testing.assert_allclose(Ob.cpu().numpy(), osr.obar(Oref, r), rtol=1e-4, atol=1e-6 / np.sqrt(ns))
    np.testing.assert_allclose(om.cpu().numpy(), (Oref * r[:, None]).mean(axis=0), rtol=1e-5, atol=1e-7)


def test_full_size_sweep_properties(cuda):
    """Config-2 sizes (8192 chains, L=64, M=256): properties that need no oracle."""
    L = lib()
    N, M, ns = 64, 256, 8192
    W, b, _ = rbm.init_normal(N, M, 0.01, seed=0)
    dev = Rbm(W, b)
    packed = torch.empty((ns, 2), dtype=torch.int32, device="cuda")
    L.call("qgx_spins_init_uniform", L.ptr(packed), ns, N, 42, L.stream_ptr())
    before = packed.clone()
    lp0, acc0 = dev.sweep(packed, 0, 1)
    assert torch.equal(packed, before) and int(acc0.sum()) == 0
    torch.testing.assert_close(lp0, dev.log_psi(packed))
    lp, acc = dev.sweep(packed, 640, 1)
    # log psi carried through 640 incremental updates equals the direct evaluation
    torch.testing.assert_close(lp, dev.log_psi(packed), rtol=0, atol=1e-4)
    a = acc.cpu().numpy()
    assert a.max() <= 640 and a.mean() > 100
    # magnetisation of the TFIM RBM with tiny weights stays close to zero on average
    s = unpack(packed, N).astype(np.float64)
    assert abs(s.mean()) < 0.05


def test_config2_slice_sweep_bit_exact(cuda):
    """A slice of the chain-64 TFIM workload (RBM 256 hidden units, N(0, 0.01^2) init): 1024
    of its 8192 chains, thermalised by the oracle for 640 proposals, then one 64-proposal
    sweep on the device, bit-exact against the oracle's Metropolis on the same Philox stream.
    (Over the 655k thermalisation proposals at this nearly flat init some accept tests fall
    within 1e-5 of a tie, where FP32 and FP64 may decide differently; the 65k proposals of
    the checked sweep have none for this seed.)"""
    N, M, ns = 64, 256, 1024
    W, b, _ = rbm.init_normal(N, M, 0.01, seed=0)
    net = rbm.RBM(W, b)
    seed = 0x5EED0C3
    therm, _, _ = metropolis.sweep(net.log_psi, metropolis.init_uniform(ns, N, 42), 640, seed, 0)
    want, want_lp, st = metropolis.sweep(net.log_psi, therm, 64, seed, 640)
    assert st["min_margin"] > 1e-5, "near-tie in the seeded case; pick another seed"
    dev = Rbm(W, b)
    packed = pack(therm)
    lp, acc = dev.sweep(packed, 64, seed, 640)
    assert (unpack(packed, N) == want).all()
    assert (acc.cpu().numpy() == st["accepts"]).all()
    np.testing.assert_allclose(lp.cpu().numpy(), want_lp, rtol=2e-6, atol=2e-5)


def test_config2_slice_eloc_and_obar(cuda):
    """Full config-2 shapes (chain 64 TFIM h = J = 1, RBM 256, 16,640 parameters) on 512
    samples: local energies and the centred, scaled Obar against the oracle."""
    L = lib()
    N, M, ns = 64, 256, 512
    W, b, _ = rbm.init_normal(N, M, 0.01, seed=0)
    net = rbm.RBM(W, b)
    s = metropolis.init_uniform(ns, N, 9)
    dev = Rbm(W, b)
    packed = pack(s)
    ops = oops.chain_tfim(N, h=1.0, J=1.0)
    op = compiled(ops)
    out = torch.empty(ns, dtype=torch.float64, device="cuda")
    L.call("qgx_rbm_eloc", L.ptr(dev.table), N, M, C.byref(op.struct), L.ptr(packed), ns, L.ptr(out), L.stream_ptr())
    want = oops.local_energy(s, ops, net.log_psi).real
    np.testing.assert_allclose(out.cpu().numpy(), want, rtol=1e-5, atol=1e-5 * np.abs(want).max())
    npar = net.nparams
    assert npar == 16640
    ws = torch.empty(L.lib().qgx_rbm_obar_workspace_bytes(N, M, ns), dtype=torch.uint8, device="cuda")
    Ob = torch.empty((ns, npar), dtype=torch.float32, device="cuda")
    om = torch.empty(npar, dtype=torch.float64, device="cuda")
    L.call("qgx_rbm_obar", L.ptr(dev.table), N, M, 0, L.ptr(packed), None, ns, L.ptr(Ob), npar, L.ptr(om),
           L.ptr(ws), ws.numel(), L.stream_ptr())
    from oracle import sr as osr
    Oref = net.jacobian(s)
    np.testing.assert_allclose(Ob.cpu().numpy(), osr.obar(Oref), rtol=1e-4, atol=1e-6 / np.sqrt(ns))
    np.testing.assert_allclose(om.cpu().numpy(), Oref.mean(axis=0), rtol=1e-5, atol=1e-7)


def test_psi_consistency_check_after_local_updates(cuda):
    """Metropolis.sweep's check (metropolis.py:201-213): log|psi| carried through the sweep's
    local updates agrees with a direct forward, so a normal sweep warns about nothing; a sweep
    whose updates ran on a perturbed copy of the table (inaccurate local updates) warns with the
    number of samples that differ when the count is read, and its samples carry the direct
    values."""
    import warnings
    import quantax_gb300 as qtx
    qtx.sites.Chain(16)
    W, b, a = rbm.init_normal(16, 32, 0.2, seed=5, visible_bias=True)
    state = qtx.state.Variational(qtx.model.RBM_Dense.from_arrays(W, b, a))
    sampler = qtx.sampler.LocalFlip(state, 128, thermal_steps=0, sweep_steps=64)
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        samples = sampler.sweep()
        assert sampler.check_local_updates() == 0
    assert torch.equal(samples.log_psi, state.log_psi_packed(samples.packed))
    model = state.model
    sweep = model.sweep
    bad = state.table.clone() * 1.05
    model.sweep = lambda table, *args: sweep(bad, *args)
    try:
        samples = sampler.sweep()
        with pytest.warns(UserWarning, match=r"\d+ out of 128 wavefunctions are not close"):
            assert sampler.check_local_updates() > 0
    finally:
        del model.sweep
    assert torch.equal(samples.log_psi, state.log_psi_packed(samples.packed))
