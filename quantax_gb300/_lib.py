"""ctypes binding of libqgx.so (the C ABI declared in include/qgx.h).

The library is built in-tree by quantax_gb300._build; there is no CPU fallback: if the
shared library is missing or no CUDA device is present, every call raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import torch

LIB_PATH = Path(__file__).resolve().parent / "libqgx.so"

QGX_OK = 0
QGX_ERR_ARG = 1
QGX_ERR_CUDA = 2
QGX_ERR_TIMEOUT = 3
QGX_ERR_NONFINITE = 4
QGX_ERR_UNSUPPORTED = 5
QGX_ERR_SOLVER = 6

PROPOSAL_LOCAL_FLIP = 0
PROPOSAL_SPIN_EXCHANGE = 1
SOLVE_SHIFT = 0
SOLVE_PINV = 1
SOLVE_SHIFT_MIXED = 2
SOLVE_SHIFT_LIB = 3
GRAM_FP32 = 0
GRAM_TF32 = 1
GRAM_BF16 = 2
GRAM_3XTF32 = 3
GRAM_FP64 = 4
CONV_FP32 = 0
CONV_TF32 = 1
CONV_BF16 = 2
CONV_GROUPED = 0x100  # OR'd into CONV_BF16: the warp-specialised kernel
RESCONV_COMPLEX = 1
RESCONV_SINHP1 = 2

vp = C.c_void_p
i32 = C.c_int32
i64 = C.c_int64
u64 = C.c_uint64
f32 = C.c_float
f64 = C.c_double


class Operator(C.Structure):
    """qgx_operator_t"""
    _fields_ = [
        ("c0", f64),
        ("n_z", i32), ("z_i", vp), ("z_J", vp),
        ("n_zz", i32), ("zz_ij", vp), ("zz_J", vp),
        ("n_f1", i32), ("f1_i", vp), ("f1_J", vp),
        ("n_f2", i32), ("f2_ij", vp), ("f2_J", vp),
    ]


class Symm(C.Structure):
    """qgx_symm_t"""
    _fields_ = [("perm", vp), ("weight", vp), ("nperm", i32), ("z2", i32)]


class RbmSweepJob(C.Structure):
    """qgx_rbm_sweep_job_t"""
    _fields_ = [
        ("table", vp), ("n", i32), ("m", i32), ("spins", vp), ("log_psi", vp), ("accepts", vp), ("ns", i64),
        ("nsteps", i32), ("proposal", i32), ("seed", u64), ("step0", u64), ("reweight", f32), ("nbr", vp),
        ("z", i32), ("hop", i32),
    ]


class RbmElocJob(C.Structure):
    """qgx_rbm_eloc_job_t"""
    _fields_ = [("table", vp), ("n", i32), ("m", i32), ("op", C.POINTER(Operator)), ("spins", vp), ("ns", i64),
                ("eloc", vp)]


RBM_BATCH_MAX_JOBS = 64  # QGX_RBM_BATCH_MAX_JOBS


# name -> (restype, argtypes)
SIGNATURES = {
    "qgx_abi_version": (C.c_int, []),
    "qgx_status_string": (C.c_char_p, [C.c_int]),
    "qgx_last_error": (C.c_char_p, []),
    "qgx_clear_last_error": (None, []),
    "qgx_philox4x32_10": (C.c_int, [vp, vp, vp, i64, vp]),
    "qgx_spins_init_uniform": (C.c_int, [vp, i64, i32, u64, vp]),
    "qgx_spins_init_fixed_up": (C.c_int, [vp, i64, i32, i32, u64, vp]),
    "qgx_spins_unpack": (C.c_int, [vp, vp, i64, i32, vp]),
    "qgx_spins_pack": (C.c_int, [vp, vp, i64, i32, vp]),
    "qgx_operator_diag": (C.c_int, [C.POINTER(Operator), vp, i64, i32, vp, vp]),
    "qgx_rbm_table_floats": (i64, [i32, i32]),
    "qgx_rbm_prepare": (C.c_int, [vp, vp, vp, i32, i32, vp, vp]),
    "qgx_rbm_log_psi": (C.c_int, [vp, i32, i32, vp, i64, vp, vp]),
    "qgx_rbm_sweep": (C.c_int, [vp, i32, i32, vp, vp, vp, i64, i32, u64, u64, f32, i32, vp, i32, i32, vp]),
    "qgx_rbm_eloc": (C.c_int, [vp, i32, i32, C.POINTER(Operator), vp, i64, vp, vp]),
    "qgx_rbm_sweep_batched": (C.c_int, [C.POINTER(RbmSweepJob), i32, C.POINTER(i32), vp]),
    "qgx_rbm_eloc_batched": (C.c_int, [C.POINTER(RbmElocJob), i32, C.POINTER(i32), vp]),
    "qgx_rbm_jacobian": (C.c_int, [vp, i32, i32, i32, vp, i64, vp, i64, vp]),
    "qgx_rbm_obar_workspace_bytes": (i64, [i32, i32, i64]),
    "qgx_rbm_obar": (C.c_int, [vp, i32, i32, i32, vp, vp, i64, vp, i64, vp, vp, i64, vp]),
    "qgx_rbm_obar_noalloc": (C.c_int, [vp, i32, i32, i32, vp, vp, i64, vp, i64, vp, vp]),
    "qgx_resconv_nparams": (i64, [i32, i32]),
    "qgx_resconv_table_floats": (i64, [i32, i32]),
    "qgx_resconv_prepare": (C.c_int, [vp, i32, i32, vp, vp]),
    "qgx_resconv_log_psi": (C.c_int, [vp, i32, i32, i32, i32, i32, vp, i64, vp, vp]),
    "qgx_resconv_sweep_workspace_bytes": (i64, [i32, i64]),
    "qgx_resconv_sweep": (C.c_int, [vp, i32, i32, i32, i32, i32, vp, vp, vp, i64, i32, u64, u64, f32, vp, i32, i32, vp,
                                    i64, vp]),
    "qgx_resconv_eloc_workspace_bytes": (i64, [i32, i64, i32]),
    "qgx_resconv_eloc": (C.c_int, [vp, i32, i32, i32, i32, i32, C.POINTER(Operator), vp, i64, vp, vp, vp, i64, vp]),
    "qgx_resconv_jacobian_workspace_bytes": (i64, [i32, i32, i32]),
    "qgx_resconv_jacobian": (C.c_int, [vp, i32, i32, i32, i32, vp, i64, vp, vp, i64, vp, i64, vp]),
    "qgx_energy_stats": (C.c_int, [vp, vp, vp, i64, vp, vp, vp, vp]),
    "qgx_reweight_factor": (C.c_int, [vp, i64, f32, vp, vp]),
    "qgx_center_columns_workspace_bytes": (i64, [i64, i64]),
    "qgx_center_columns": (C.c_int, [vp, i64, i64, i64, vp, vp, vp, i64, vp]),
    "qgx_gram": (C.c_int, [vp, i64, i64, i64, vp, i64, i32, vp]),
    "qgx_gram_t": (C.c_int, [vp, i64, i64, i64, vp, i64, vp]),
    "qgx_gram_tc": (C.c_int, [vp, i32, i64, i64, i64, vp, i64, vp, vp]),
    "qgx_f32_to_bf16": (C.c_int, [vp, i64, i64, i64, vp, i64, vp]),
    "qgx_solve_workspace_bytes": (C.c_int, [i64, i64, i32, C.POINTER(i64)]),
    "qgx_minsr_solve": (C.c_int, [vp, i64, vp, i64, i64, vp, i32, f64, f64, f64, f64, f64, vp, vp, vp, i64, vp]),
    "qgx_last_solve_kernels": (i64, []),
    "qgx_transpose": (C.c_int, [vp, i64, i64, i64, vp, i64, i32, vp]),
    "qgx_obar_matvec": (C.c_int, [vp, i64, i64, i64, vp, vp, vp]),
    "qgx_scale_columns": (C.c_int, [vp, i64, i64, i64, vp, vp]),
    "qgx_exact_draw": (C.c_int, [vp, i64, i64, u64, u64, vp, vp]),
    "qgx_csr_matvec": (C.c_int, [vp, vp, vp, i64, vp, i32, vp, vp]),
    "qgx_er_weight_rows": (C.c_int, [vp, i64, i64, i64, vp, i32, vp]),
    "qgx_er_center": (C.c_int, [vp, i64, i64, i64, vp, i32, vp, vp]),
    "qgx_resconv_log_psi_symm_workspace_bytes": (i64, [i32, i64, i32]),
    "qgx_resconv_log_psi_symm": (C.c_int, [vp, i32, i32, i32, i32, i32, C.POINTER(Symm), vp, i64, vp, vp, i64, vp]),
    "qgx_resconv_sweep_symm_workspace_bytes": (i64, [i32, i64, i32]),
    "qgx_resconv_sweep_symm": (C.c_int, [vp, i32, i32, i32, i32, i32, C.POINTER(Symm), vp, vp, vp, i64, i32, u64, u64,
                                         f32, vp, i32, i32, vp, i64, vp]),
    "qgx_resconv_eloc_symm_workspace_bytes": (i64, [i32, i64, i32, i32]),
    "qgx_resconv_eloc_symm": (C.c_int, [vp, i32, i32, i32, i32, i32, C.POINTER(Symm), C.POINTER(Operator), vp, i64,
                                        vp, vp, vp, i64, vp]),
    "qgx_resconv_jacobian_symm_workspace_bytes": (i64, [i32, i32, i32, i64, i32]),
    "qgx_resconv_jacobian_symm": (C.c_int, [vp, i32, i32, i32, i32, C.POINTER(Symm), vp, i64, vp, vp, i64, vp, i64,
                                            vp]),
    "qgx_rbm_log_psi_symm_workspace_bytes": (i64, [i32, i64, i32]),
    "qgx_rbm_log_psi_symm": (C.c_int, [vp, i32, i32, C.POINTER(Symm), vp, i64, vp, vp, i64, vp]),
    "qgx_rbm_sweep_symm_workspace_bytes": (i64, [i32, i64, i32]),
    "qgx_rbm_sweep_symm": (C.c_int, [vp, i32, i32, C.POINTER(Symm), vp, vp, vp, i64, i32, u64, u64, f32, i32, vp, i32,
                                     i32, vp, i64, vp]),
    "qgx_rbm_eloc_symm_workspace_bytes": (i64, [i32, i64, i32, i32]),
    "qgx_rbm_eloc_symm": (C.c_int, [vp, i32, i32, C.POINTER(Symm), C.POINTER(Operator), vp, i64, vp, vp, vp, i64,
                                    vp]),
    "qgx_rbm_jacobian_symm_workspace_bytes": (i64, [i32, i32, i32, i64, i32]),
    "qgx_rbm_jacobian_symm": (C.c_int, [vp, i32, i32, i32, C.POINTER(Symm), vp, i64, vp, vp, i64, vp, i64, vp]),
    "qgx_rbm_conv_table_floats": (i64, [i32, i32, i32]),
    "qgx_rbm_conv_prepare": (C.c_int, [vp, i32, i32, i32, vp, vp]),
    "qgx_rbm_conv_jacobian": (C.c_int, [vp, i32, i32, i32, vp, i64, vp, i64, vp]),
    "qgx_column_sumsq_workspace_bytes": (i64, [i64, i64]),
    "qgx_column_sumsq": (C.c_int, [vp, i64, i64, i64, vp, vp, i64, vp]),
    "qgx_obar_rmatvec_workspace_bytes": (C.c_int, [i64, i64, vp]),
    "qgx_obar_rmatvec": (C.c_int, [vp, i64, i64, i64, vp, vp, vp, i64, vp]),
    "qgx_sym_solve": (C.c_int, [vp, i64, vp, i32, f64, f64, f64, f64, vp, vp, vp, i64, vp]),
    "qgx_sr_solve": (C.c_int, [vp, i64, vp, i64, i64, vp, i32, f64, f64, f64, f64, f64, vp, vp, vp, i64, vp]),
    "qgx_apply_update": (C.c_int, [vp, vp, i64, vp, vp]),
    "qgx_log_psi_mismatch": (C.c_int, [vp, vp, i64, vp, vp, vp]),
    "qgx_cholesky_workspace_bytes": (i64, [i64]),
    "qgx_cholesky": (C.c_int, [vp, i64, i64, vp, vp, vp, i64, vp]),
}


class QgxError(RuntimeError):
    def __init__(self, name, status, lib):
        self.status = status
        msg = lib.qgx_status_string(status).decode()
        detail = lib.qgx_last_error().decode()  # cleared before the call: this call's reason, if any
        super().__init__(f"{name} failed: {msg} ({status}) {detail}".strip())


# qgx kernels each entry point launches (library calls such as cuSOLVER not counted)
KERNELS_PER_CALL = {
    "qgx_philox4x32_10": 1, "qgx_spins_init_uniform": 1, "qgx_spins_init_fixed_up": 1, "qgx_spins_unpack": 1,
    "qgx_spins_pack": 1, "qgx_operator_diag": 1, "qgx_rbm_prepare": 1, "qgx_rbm_log_psi": 1, "qgx_rbm_sweep": 1,
    "qgx_rbm_eloc": 1, "qgx_rbm_jacobian": 1, "qgx_rbm_obar": 4, "qgx_rbm_obar_noalloc": 4, "qgx_resconv_prepare": 2,
    "qgx_resconv_log_psi": 1, "qgx_resconv_eloc": 6, "qgx_resconv_log_psi_symm": 3, "qgx_resconv_eloc_symm": 10,
    "qgx_resconv_jacobian_symm": 4, "qgx_rbm_log_psi_symm": 3, "qgx_rbm_eloc_symm": 10,
    "qgx_resconv_jacobian": 1, "qgx_energy_stats": 1, "qgx_reweight_factor": 1,
    "qgx_gram": 1, "qgx_gram_t": 1, "qgx_gram_tc": 1, "qgx_f32_to_bf16": 1, "qgx_transpose": 1, "qgx_obar_matvec": 1, "qgx_obar_rmatvec": 2, "qgx_rbm_conv_prepare": 1, "qgx_column_sumsq": 2,
    "qgx_rbm_conv_jacobian": 1, "qgx_apply_update": 2, "qgx_csr_matvec": 1, "qgx_er_weight_rows": 1, "qgx_exact_draw": 1,
    "qgx_er_center": 1, "qgx_log_psi_mismatch": 1,
}
launch_count = 0


def _kernels(name, args):
    if name in ("qgx_minsr_solve", "qgx_sr_solve", "qgx_sym_solve"):
        return int(lib().qgx_last_solve_kernels())
    if name == "qgx_center_columns":  # partial sums, reduction, mean split, centring
        return 4 if int(args[1]) > 0 else 0
    if name == "qgx_scale_columns":
        return 1 + (int(args[1]) - 1) // 65535 if int(args[1]) > 0 and int(args[2]) > 0 else 0
    if name in ("qgx_rbm_sweep_batched", "qgx_rbm_eloc_batched"):  # the count the call reports
        return int(args[2]._obj.value) if args[2] is not None else 0
    if name == "qgx_resconv_sweep":
        return 2 + 3 * int(args[10])  # step base, forward, then propose / forward / accept per step
    if name == "qgx_resconv_sweep_symm":
        return 4 + 5 * int(args[11])  # each forward is expand / forward / combine
    if name == "qgx_rbm_sweep_symm":
        return 4 + 5 * int(args[8])
    if name == "qgx_rbm_jacobian_symm":  # the projected forward, then per chunk of samples the rows and their sum
        n, m, vb, ns = int(args[1]), int(args[2]), int(args[3]), int(args[6])
        sym = args[4]._obj
        nsymm = sym.nperm * (2 if sym.z2 else 1)
        npar = m * n + m + (n if vb else 0)
        cs = max(1, min(min(ns, 65535), (1 << 26) // (nsymm * npar)))
        return 3 + 2 * ((ns + cs - 1) // cs) if ns > 0 else 0
    return KERNELS_PER_CALL.get(name, 0)


_LIB = None


def load(path: Path | None = None):
    """Load libqgx.so and bind every entry point (does not need a GPU)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with quantax_gb300._build.build() "
                           "(the qgx CUDA library has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def lib():
    return load()


def call(name, *args):
    """Call an entry point that returns a status code; raise on failure."""
    global launch_count
    L = load()
    L.qgx_clear_last_error()
    rc = getattr(L, name)(*args)
    if rc != QGX_OK:
        raise QgxError(name, rc, L)
    launch_count += _kernels(name, args)


def ptr(t: torch.Tensor | None):
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("qgx kernels take CUDA tensors")
    return C.c_void_p(t.data_ptr())


def stream_ptr(stream: torch.cuda.Stream | None = None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("quantax_gb300 runs on a CUDA GPU (sm_103a); no device is available "
                           "and there is no CPU fallback")
