"""SPRING, MARCH and AdamSR (quantax/optimizer/sr.py:198-429) against the oracle's
restatement: four consecutive solves on fresh seeded Obar / Ebar, through both solve branches
(MinSR, Ns < Np, and SR, Ns >= Np), plus the save / load round trip of the momentum state.

Tolerance: 1e-4 relative 2-norm per step. The device builds the Gram of the FP32 Obar with FP32
products (the oracle in FP64) and the momentum terms carry that error forward."""
import numpy as np
import pytest
import torch

from oracle import sr as osr

pytestmark = pytest.mark.gpu

RSHIFT, ASHIFT, TOL = 1e-6, 1e-3, 1e-4


def _state():
    import quantax_gb300 as qtx
    qtx.set_default_dtype(np.float64)
    qtx.sites.Chain(8)
    qtx.set_random_seed(1)
    return qtx.state.Variational(qtx.model.RBM_Dense(16, init_std=0.01)), qtx.operator.Ising(h=1.0)


def _make(kind, file=None):
    import quantax_gb300 as qtx
    state, H = _state()
    solver = qtx.optimizer.auto_shift_eig(rshift=RSHIFT, ashift=ASHIFT)
    cls = getattr(qtx.optimizer, kind)
    return cls(state, H, solver=solver, file=file)


def _inputs(rng, ns, np_):
    A = (rng.normal(size=(ns, np_)) / np.sqrt(np_)).astype(np.float32)
    b = rng.normal(size=ns)
    return A, b


def _oracle_solver(A, b):
    if A.shape[0] < A.shape[1]:
        return osr.minnorm_shift(A, b, rshift=RSHIFT, ashift=ASHIFT)
    return osr.lstsq_shift(A, b, rshift=RSHIFT, ashift=ASHIFT)


class _Oracle:
    def __init__(self, kind, np_):
        self.kind, self.t = kind, 0
        self.last = np.zeros(np_)
        self.V = np.zeros(np_)
        self.m = np.zeros(np_)
        self.v = np.zeros(np_)

    def step(self, A, b):
        A = A.astype(np.float64)
        if self.kind == "SPRING":
            self.last = osr.spring_step(A, b, self.last, 0.9, _oracle_solver)
            return self.last
        self.t += 1
        if self.kind == "MARCH":
            self.last, self.V = osr.march_step(A, b, self.last, self.V, self.t, 0.95, 0.995, _oracle_solver)
            return self.last
        x, self.m, self.v = osr.adamsr_step(A, b, self.m, self.v, self.t, 0.95, 0.995, _oracle_solver)
        return x


def _dev_step(opt, A, b):
    return opt.solve(torch.as_tensor(A).cuda(), torch.as_tensor(b).cuda()).cpu().numpy()


@pytest.mark.parametrize("kind", ["SPRING", "MARCH", "AdamSR"])
@pytest.mark.parametrize("ns", [64, 600])
def test_momentum_sr_steps(cuda, kind, ns):
    opt = _make(kind)
    np_ = opt.state.nparams
    ref = _Oracle(kind, np_)
    rng = np.random.default_rng(ns + len(kind))
    for it in range(4):
        A, b = _inputs(rng, ns, np_)
        x = _dev_step(opt, A, b)
        xr = ref.step(A, b)
        err = np.linalg.norm(x - xr) / np.linalg.norm(xr)
        assert err < TOL, (kind, ns, it, err)


@pytest.mark.parametrize("kind", ["SPRING", "MARCH", "AdamSR"])
def test_momentum_sr_save_load(cuda, kind, tmp_path):
    """Two steps, save, a new optimizer loads the file: its next step equals the original's."""
    opt = _make(kind)
    np_ = opt.state.nparams
    rng = np.random.default_rng(7)
    for _ in range(2):
        _dev_step(opt, *_inputs(rng, 64, np_))
    f = tmp_path / f"{kind}.eqx"
    opt.save(f)
    A, b = _inputs(rng, 64, np_)
    restored = _make(kind, file=f)
    x1 = _dev_step(opt, A, b)
    x2 = _dev_step(restored, A, b)
    assert np.array_equal(x1, x2)


def test_obar_matvec_and_scale_columns(cuda):
    """qgx_obar_matvec (FP64 accumulation) and qgx_scale_columns on a padded row stride."""
    from quantax_gb300 import _lib as L
    rng = np.random.default_rng(2)
    rows, cols, lda = 70000, 37, 40  # more rows than one grid dimension of the scaling launch
    buf = torch.as_tensor(rng.normal(size=(rows, lda)).astype(np.float32)).cuda()
    A = buf[:, :cols]
    x = rng.normal(size=cols)
    y = torch.empty(rows, dtype=torch.float64, device="cuda")
    xd = torch.as_tensor(x).cuda()
    L.call("qgx_obar_matvec", L.ptr(A), rows, cols, lda, L.ptr(xd), L.ptr(y), L.stream_ptr())
    An = A.cpu().numpy().astype(np.float64)
    np.testing.assert_allclose(y.cpu().numpy(), An @ x, rtol=1e-12, atol=1e-12)
    s = rng.uniform(0.5, 2.0, size=cols)
    pad_before = buf[:, cols:].clone()
    sd = torch.as_tensor(s).cuda()
    L.call("qgx_scale_columns", L.ptr(A), rows, cols, lda, L.ptr(sd), L.stream_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(A.cpu().numpy(), (An * s[None, :]).astype(np.float32))
    assert torch.equal(buf[:, cols:], pad_before)
