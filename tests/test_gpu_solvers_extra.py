"""The remaining solver factories of quantax/optimizer/solver.py against the oracle:
sgd_solver, lstsq_shift_cg, block_pinv_eig, minsr_pinv_eig."""
import numpy as np
import pytest
import torch

from oracle import sr as osr

pytestmark = pytest.mark.gpu


def _rbm_opt(solver):
    import quantax_gb300 as qtx
    qtx.set_default_dtype(np.float64)
    qtx.sites.Chain(8)
    qtx.set_random_seed(1)
    state = qtx.state.Variational(qtx.model.RBM_Dense(16, init_std=0.01))
    return qtx.optimizer.SR(state, qtx.operator.Ising(h=1.0), solver=solver)


def _Ab(ns, np_, seed):
    rng = np.random.default_rng(seed)
    return (rng.normal(size=(ns, np_)) / np.sqrt(ns)).astype(np.float32), rng.normal(size=ns)


def test_sgd_solver(cuda):
    import quantax_gb300 as qtx
    opt = _rbm_opt(qtx.optimizer.sgd_solver())
    A, b = _Ab(300, 144, 0)
    x = opt.solve(torch.as_tensor(A).cuda(), torch.as_tensor(b).cuda()).cpu().numpy()
    np.testing.assert_allclose(x, osr.sgd(A.astype(np.float64), b), rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("ns", [600, 100])
def test_lstsq_shift_cg(cuda, ns):
    """CG to rtol 1e-10 reaches the direct solution of (S + 0.01 diag S) x = A^T b (stated:
    1e-7 relative; the CG stops on the residual). Also with fewer samples than parameters,
    where the relative shift alone regularises S."""
    import quantax_gb300 as qtx
    opt = _rbm_opt(qtx.optimizer.lstsq_shift_cg(diag_shift=0.01, rtol=1e-10))
    A, b = _Ab(ns, 144, ns)
    x = opt.solve(torch.as_tensor(A).cuda(), torch.as_tensor(b).cuda()).cpu().numpy()
    ref = osr.lstsq_shift_direct(A.astype(np.float64), b, 0.01)
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-7
    # the default tolerance stops earlier but stays close
    opt2 = _rbm_opt(qtx.optimizer.lstsq_shift_cg())
    x2 = opt2.solve(torch.as_tensor(A).cuda(), torch.as_tensor(b).cuda()).cpu().numpy()
    assert np.linalg.norm(x2 - ref) / np.linalg.norm(ref) < 1e-3


def test_block_pinv_eig_resconv_layers(cuda):
    """ResConv(2 blocks, 8 channels) on 4 x 4: the layers are its two residual blocks
    (param_blocks: 664 and 1160 parameters); per-layer pinv of Obar against the oracle. Stated:
    1e-6 relative on the MinSR branch (FP64 T from FP32 Obar) and 1e-5 on the SR branch, whose
    S = Obar^T Obar is the default FP32-accumulated Gram (as the SR-branch Gram test states)."""
    import quantax_gb300 as qtx
    qtx.set_default_dtype(np.float64)
    qtx.sites.Square(4, Nparticles=(8, 8))
    qtx.set_random_seed(2)
    state = qtx.state.Variational(qtx.model.ResConv(2, 8))
    solver = qtx.optimizer.block_pinv_eig(state, rtol=1e-10)
    blocks = list(solver.blocks)
    assert blocks == state.model.param_blocks() and sum(blocks) == state.nparams
    opt = qtx.optimizer.SR(state, qtx.operator.Heisenberg(msr=True), solver=solver)
    for ns in (200, 2000):  # MinSR and SR branches inside the blocks
        A, b = _Ab(ns, state.nparams, ns + 1)
        x = opt.solve(torch.as_tensor(A).cuda(), torch.as_tensor(b).cuda()).cpu().numpy()
        ref = osr.block_pinv(A.astype(np.float64), b, blocks, rtol=1e-10)
        assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < (1e-6 if ns < state.nparams else 1e-5), ns


def test_minsr_pinv_eig(cuda):
    import quantax_gb300 as qtx
    rng = np.random.default_rng(4)
    M = rng.normal(size=(120, 90))
    T = M @ M.T  # rank 90: the soft inverse cuts the null space
    b = rng.normal(size=120)
    solver = qtx.optimizer.minsr_pinv_eig(rtol=1e-8)
    Td = torch.as_tensor(T).cuda()
    x = solver(Td, torch.as_tensor(b).cuda()).cpu().numpy()
    assert torch.equal(Td.cpu(), torch.as_tensor(T))
    ref = osr.minsr_pinv(T, b, rtol=1e-8)
    np.testing.assert_allclose(x, ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max())
    with pytest.raises(NotImplementedError):
        qtx.optimizer.minsr_pinv_eig(tol_snr=1.0)
