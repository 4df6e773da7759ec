"""The C ABI boundary and the host-side logic, without a GPU."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import lattice, operators as oops

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "qgx.h"


def header_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qgx_\w+)\s*\(", text)))


def test_library_exports_every_header_symbol(qgx_built):
    names = header_functions()
    assert len(names) >= 25
    lib = ctypes.CDLL(str(qgx_built))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(qgx_built)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(qgx_\w+)\b", out))
    assert set(names) <= exported


def test_python_binding_covers_header(qgx_built):
    from quantax_gb300 import _lib
    assert set(header_functions()) == set(_lib.SIGNATURES)
    L = _lib.load()
    assert L.qgx_abi_version() == 1
    assert L.qgx_status_string(0) == b"ok"
    # size queries need no device
    assert L.qgx_rbm_table_floats(64, 256) == 3 * 64 * 256 + 256 + 64
    assert L.qgx_rbm_obar_workspace_bytes(64, 256, 8192) > 8192 * 256 * 4
    assert L.qgx_center_columns_workspace_bytes(100, 10) > 0


def test_argument_errors_are_reported_without_a_device(qgx_built):
    from quantax_gb300 import _lib
    L = _lib.load()
    # negative sizes and null pointers are rejected before any CUDA call
    assert L.qgx_spins_init_uniform(None, -1, 8, 1, None) == _lib.QGX_ERR_ARG
    assert L.qgx_rbm_sweep(None, 8, 16, None, None, None, 4, 1, 0, 0, 2.0, 7, None, 0, 1, None) == _lib.QGX_ERR_ARG
    assert L.qgx_gram(None, 4, 4, 2, None, 4, 0, None) == _lib.QGX_ERR_ARG
    assert L.qgx_spins_init_uniform(None, 0, 8, 1, None) == _lib.QGX_OK  # empty batch is a no-op
    # exact sampling and exact reconfiguration entry points
    assert L.qgx_exact_draw(None, 0, 4, 1, 0, None, None) == _lib.QGX_ERR_ARG  # empty basis
    assert L.qgx_exact_draw(None, 8, 4, 1, 0, None, None) == _lib.QGX_ERR_ARG  # null pointers
    assert L.qgx_exact_draw(None, 8, 0, 1, 0, None, None) == _lib.QGX_OK       # no samples
    assert L.qgx_csr_matvec(None, None, None, 4, None, 3, None, None) == _lib.QGX_ERR_ARG  # nvec not 1 or 2
    assert L.qgx_csr_matvec(None, None, None, 4, None, 1, None, None) == _lib.QGX_ERR_ARG
    assert L.qgx_er_weight_rows(None, 4, 8, 4, None, 0, None) == _lib.QGX_ERR_ARG  # ldo < cols
    assert L.qgx_er_center(None, 4, 8, 8, None, 1, None, None) == _lib.QGX_ERR_ARG
    assert L.qgx_column_sumsq(None, 4, 8, 4, None, None, 0, None) == _lib.QGX_ERR_ARG
    # the projected RBM: a missing or malformed group, sizes past the kernels' limits, an
    # unknown proposal, SpinExchange without a neighbour table
    import ctypes as C
    perm = (C.c_int16 * 16)(*range(16))
    w = (C.c_double * 2)(1.0, 0.0)
    sym = _lib.Symm(C.cast(perm, C.c_void_p), C.cast(w, C.c_void_p), 1, 0)
    bad = _lib.Symm(None, C.cast(w, C.c_void_p), 1, 0)
    assert L.qgx_rbm_log_psi_symm(None, 16, 32, None, None, 4, None, None, 0, None) == _lib.QGX_ERR_ARG
    assert L.qgx_rbm_log_psi_symm(None, 16, 32, C.byref(bad), None, 4, None, None, 0, None) == _lib.QGX_ERR_ARG
    assert L.qgx_rbm_log_psi_symm(None, 300, 32, C.byref(sym), None, 4, None, None, 0, None) == _lib.QGX_ERR_ARG
    assert L.qgx_rbm_log_psi_symm(None, 16, 32, C.byref(sym), None, 0, None, None, 0, None) == _lib.QGX_OK
    assert L.qgx_rbm_sweep_symm(None, 16, 32, C.byref(sym), None, None, None, 4, 1, 0, 0, 2.0, 7, None, 0, 1,
                                None, 0, None) == _lib.QGX_ERR_ARG
    assert L.qgx_rbm_sweep_symm(None, 16, 32, C.byref(sym), None, None, None, 4, 1, 0, 0, 2.0,
                                _lib.PROPOSAL_SPIN_EXCHANGE, None, 0, 1, None, 0, None) == _lib.QGX_ERR_ARG
    assert L.qgx_rbm_jacobian_symm(None, 16, 32, 0, C.byref(sym), None, 4, None, None, 100, None, 0,
                                   None) == _lib.QGX_ERR_ARG  # ldo below the 560 parameters
    assert L.qgx_rbm_log_psi_symm_workspace_bytes(16, 4, 1) > 0


def test_no_cpu_fallback_without_library(tmp_path):
    from quantax_gb300 import _lib
    with pytest.raises(RuntimeError, match="missing"):
        _lib.load(tmp_path / "libqgx.so")


def test_sites_match_oracle():
    import quantax_gb300 as qtx
    sq = qtx.sites.Square(10, Nparticles=(50, 50))
    for o in (1, 2):
        np.testing.assert_array_equal(sq.get_neighbor(o), lattice.neighbors((10, 10), o))
    np.testing.assert_array_equal(sq.neighbor_table(1), lattice.neighbor_table((10, 10), 1))
    ch = qtx.sites.Chain(8)
    np.testing.assert_array_equal(ch.get_neighbor(), lattice.neighbors((8,), 1))


@pytest.mark.parametrize("case", ["tfim8", "heis16", "j1j2_16"])
def test_operator_compiler_matches_oracle_matrix(case):
    import quantax_gb300 as qtx
    if case == "tfim8":
        qtx.sites.Chain(8)
        H = qtx.operator.Ising(h=0.7, J=1.3)
        ref = oops.ising_op_list(8, lattice.neighbors((8,), 1), 0.7, 1.3)
        nup = None
    elif case == "heis16":
        qtx.sites.Square(4, Nparticles=(8, 8))
        H = qtx.operator.Heisenberg(msr=True)
        ref = oops.heisenberg_op_list(lattice.neighbors((4, 4), [1]), [1.0], [1], True)
        nup = 8
    else:
        qtx.sites.Square(4, Nparticles=(8, 8))
        H = qtx.operator.Heisenberg(J=[1, 0.5], n_neighbor=[1, 2], msr=True)
        ref = oops.square_j1j2(4, 0.5, True)
        nup = 8
    n = qtx.get_sites().N
    A = H.to_sparse(nup).toarray()
    B = oops.sparse_matrix(n, ref, nup)[0].toarray()
    np.testing.assert_allclose(A, B, atol=1e-12)


def test_operator_compiler_rejects_unsupported():
    import quantax_gb300 as qtx
    qtx.sites.Chain(4)
    with pytest.raises(NotImplementedError):
        qtx.operator.compile_op_list([["xxx", [[1.0, 0, 1, 2]]]])
    with pytest.raises(NotImplementedError):
        qtx.operator.compile_op_list([["zx", [[1.0, 0, 1]]]])


def test_solver_descriptors():
    from quantax_gb300 import optimizer as opt
    s = opt.auto_shift_eig(ashift=1e-4)
    assert s.kind == "shift" and s.use_minnorm(10, 20) and not s.use_minnorm(20, 10)
    assert opt.minnorm_pinv_eig().use_minnorm(30, 20)
    assert not opt.lstsq_pinv_eig().use_minnorm(10, 20)


def test_serving_job_stream_and_estimates():
    from quantax_gb300.serving import JobSpec, poisson_jobs
    jobs = poisson_jobs(20, seed=3)
    assert len(jobs) == 20 and all(a.arrival < b.arrival for a, b in zip(jobs, jobs[1:]))
    assert {j.kind for j in jobs} == {"tfim", "j1j2"}
    # the parameter count formula matches the ResConv oracle's
    from oracle import resconv
    j = JobSpec("x", "j1j2", 6, 1024, 1, 0, blocks=5, channels=12)
    assert j.nparams() == resconv.nparams(5, 12)
    t = JobSpec("y", "tfim", 64, 8192, 1, 0, alpha=4)
    assert t.nparams() == 256 * 64 + 256
    assert t.hbm_bytes() > 8192 * 16640 * 4 + 8192 * 8192 * 8
