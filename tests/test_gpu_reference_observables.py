"""The CUDA local-estimator path against operators pinned to the reference's printed values.

tests/test_reference_observables.py pins the oracle's operator matrices (the Ising chain of
ops with the magnetisation M2 = M @ M, and the Heisenberg model with its spin correlations)
to values that tutorials/samples.ipynb and tutorials/exact_diag.ipynb print. Here the same
observables go through the device path a user calls, Operator.Oloc on the GPU, for an RBM
state summed over every configuration of the basis: sum_s |psi(s)|^2 O_loc(s) / sum_s |psi|^2
must equal psi^T O psi / psi^T psi built from the pinned oracle matrix and the oracle's FP64
amplitudes of the same RBM, to 1e-5 of the |psi|^2-weighted mean of |O_loc| (the FP32 scale;
the mean itself can cancel far below it). The CUDA tables, their diagonal / flip conventions
and the psi(s')/psi(s) ratios are thereby pinned to the reference itself.
"""
import numpy as np
import pytest
import torch

from oracle import lattice, operators as ops, rbm

pytestmark = pytest.mark.gpu
N = 16


def _all_configs(nup=None):
    codes = np.arange(1 << N, dtype=np.int64)
    if nup is not None:
        pop = sum((codes >> i) & 1 for i in range(N))
        codes = codes[pop == nup]
    return codes, (((codes[:, None] >> np.arange(N)) & 1) * 2 - 1).astype(np.int8)


def _exact_gpu(qtx, state, op, spins):
    from quantax_gb300.sampler import Samples
    from quantax_gb300.state import pack_spins
    packed = pack_spins(spins, N)
    lp = state.log_psi_packed(packed)
    lpr = (lp.real if lp.is_complex() else lp).double()
    E = op.Oloc(state, Samples(packed, lp, N, None))
    E = E.real if E.is_complex() else E
    w = torch.exp(2.0 * (lpr - lpr.max()))
    # the mean and the |psi|^2-weighted mean magnitude of the local values (the scale of the
    # FP32 errors: the mean itself can cancel to well below it)
    return float((w * E).sum() / w.sum()), float((w * E.abs()).sum() / w.sum())


def _exact_oracle(net, mat, spins):
    lp = net.log_psi(spins).real
    psi = np.exp(lp - lp.max())
    return float(psi @ (mat @ psi) / (psi @ psi))


def _state(qtx, seed):
    W, b, a = rbm.init_normal(N, 16, 0.25, seed=seed, visible_bias=True)
    return qtx.state.Variational(qtx.model.RBM_Dense.from_arrays(W, b, a)), rbm.RBM(W, b, a)


def test_gpu_ising_magnetisation_and_energy(cuda):
    import quantax_gb300 as qtx
    from quantax_gb300.operator import sigma_z
    qtx.sites.Square(4)
    state, net = _state(qtx, 21)
    _, spins = _all_configs()
    M = sum(sigma_z(i) for i in range(N)) / N
    M2_oracle = ops.sparse_matrix(N, [["zz", [[4.0 / N ** 2, i, j] for i in range(N) for j in range(N)]]])[0]
    (got, scale), want = _exact_gpu(qtx, state, M @ M, spins), _exact_oracle(net, M2_oracle, spins)
    assert abs(got - want) < 1e-5 * scale
    H_oracle, _ = ops.sparse_matrix(N, ops.ising_op_list(N, lattice.neighbors((4, 4), 1), 3.0, 1.0))
    (got, scale), want = _exact_gpu(qtx, state, qtx.operator.Ising(h=3.0), spins), _exact_oracle(net, H_oracle, spins)
    assert abs(got - want) < 1e-5 * scale


@pytest.mark.parametrize("j", [1, 2])
def test_gpu_heisenberg_correlation_and_energy(cuda, j):
    import quantax_gb300 as qtx
    from quantax_gb300.operator import sigma_m, sigma_p, sigma_z
    qtx.sites.Square(4, Nparticles=(8, 8))
    state, net = _state(qtx, 30 + j)
    _, spins = _all_configs(nup=8)
    C = (sigma_z(0) @ sigma_z(j) + 2 * sigma_p(0) @ sigma_m(j) + 2 * sigma_m(0) @ sigma_p(j)) / 4
    C_oracle, _ = ops.sparse_matrix(N, [["zz", [[1.0, 0, j]]], ["+-", [[0.5, 0, j]]], ["-+", [[0.5, 0, j]]]], nup=8)
    (got, scale), want = _exact_gpu(qtx, state, C, spins), _exact_oracle(net, C_oracle, spins)
    assert abs(got - want) < 1e-5 * scale
    H_oracle, _ = ops.sparse_matrix(N, ops.heisenberg_op_list([lattice.neighbors((4, 4), 1)]), nup=8)
    (got, scale), want = _exact_gpu(qtx, state, qtx.operator.Heisenberg(), spins), _exact_oracle(net, H_oracle, spins)
    assert abs(got - want) < 1e-5 * scale
    qtx.sites.Square(4)
