"""Time one qgx kernel on synthetic data (the command line behind the profiles).

    python -m quantax_gb300.kernel_bench gram --mode tf32 --rows 2048 --k 16640 --reps 3
    python -m quantax_gb300.kernel_bench sweep --ns 8192 --n 64 --m 256 --steps 64
    python -m quantax_gb300.kernel_bench eloc --ns 8192 --n 64 --m 256
    python -m quantax_gb300.kernel_bench obar --ns 8192 --n 64 --m 256
    python -m quantax_gb300.kernel_bench rc_forward --ns 16384 --L 10 --blocks 8 --channels 16 --conv bf16
    python -m quantax_gb300.kernel_bench rc_sweep --ns 16384 --steps 4
    python -m quantax_gb300.kernel_bench rc_eloc --ns 16384
    python -m quantax_gb300.kernel_bench rc_jacobian --ns 2048
    python -m quantax_gb300.kernel_bench chol --rows 8192 --k 16640 --reps 3 [--lib]
    python -m quantax_gb300.kernel_bench dgemm --rows 8192 --reps 3

Prints one JSON line with the mean device time per launch (CUDA events, after warm-up).
"""
from __future__ import annotations

import argparse
import json

import numpy as np
import torch

from . import _build, _lib as L


def _events(fn, reps, warmup=2):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _rbm(n, m, ns, seed=0):
    rng = np.random.default_rng(seed)
    W = torch.as_tensor(rng.normal(0, 0.01, (m, n)).astype(np.float32)).cuda()
    b = torch.as_tensor(rng.normal(0, 0.01, m).astype(np.float32)).cuda()
    table = torch.empty(L.lib().qgx_rbm_table_floats(n, m), dtype=torch.float32, device="cuda")
    L.call("qgx_rbm_prepare", L.ptr(W), L.ptr(b), None, n, m, L.ptr(table), L.stream_ptr())
    spins = torch.empty((ns, (n + 31) // 32), dtype=torch.int32, device="cuda")
    L.call("qgx_spins_init_uniform", L.ptr(spins), ns, n, 5, L.stream_ptr())
    return table, spins


def _resconv(a, st):
    import ctypes as C
    import quantax_gb300 as qtx
    Ls, B, Cc, ns = a.L, a.blocks, a.channels, a.ns
    n = Ls * Ls
    npar = int(L.lib().qgx_resconv_nparams(B, Cc))
    rng = np.random.default_rng(0)
    params = torch.as_tensor(rng.normal(0, 0.1, npar).astype(np.float32)).cuda()
    table = torch.empty(L.lib().qgx_resconv_table_floats(B, Cc), dtype=torch.float32, device="cuda")
    L.call("qgx_resconv_prepare", L.ptr(params), B, Cc, L.ptr(table), st)
    spins = torch.empty((ns, (n + 31) // 32), dtype=torch.int32, device="cuda")
    L.call("qgx_spins_init_fixed_up", L.ptr(spins), ns, n, n // 2, 5, st)
    flop_fwd = 2.0 * n * 9 * Cc * (1 + (2 * B - 1) * Cc)  # 2 x MACs per forward
    prec = {"fp32": L.CONV_FP32, "tf32": L.CONV_TF32, "bf16": L.CONV_BF16,
            "bf16_grouped": L.CONV_BF16 | L.CONV_GROUPED}[a.conv]
    res = dict(ns=ns, L=Ls, blocks=B, channels=Cc, conv=a.conv, flop_per_forward=flop_fwd)
    if a.kernel == "rc_forward":
        lp = torch.empty((ns, 2), dtype=torch.float32, device="cuda")
        fn = lambda: L.call("qgx_resconv_log_psi", L.ptr(table), Ls, B, Cc, 1, prec, L.ptr(spins), ns, L.ptr(lp), st)
        ms = _events(fn, a.reps)
        res.update(ms=ms, forwards_per_s=ns / ms * 1e3, tflops=flop_fwd * ns / ms / 1e9)
    elif a.kernel == "rc_sweep":
        qtx.sites.Square(Ls, Nparticles=(n // 2, n // 2))
        nbr = torch.as_tensor(qtx.get_sites().neighbor_table(1)).cuda()
        lp = torch.empty((ns, 2), dtype=torch.float32, device="cuda")
        ws = torch.empty(L.lib().qgx_resconv_sweep_workspace_bytes(Ls, ns), dtype=torch.uint8, device="cuda")
        fn = lambda: L.call("qgx_resconv_sweep", L.ptr(table), Ls, B, Cc, 1, prec, L.ptr(spins), L.ptr(lp), None, ns,
                            a.steps, 7, 0, 2.0, L.ptr(nbr), nbr.shape[1], 1, L.ptr(ws), ws.numel(), st)
        ms = _events(fn, a.reps)
        res.update(steps=a.steps, ms=ms, proposals_per_s=ns * a.steps / ms * 1e3,
                   tflops=flop_fwd * ns * (a.steps + 1) / ms / 1e9)
    elif a.kernel == "rc_eloc":
        qtx.sites.Square(Ls, Nparticles=(n // 2, n // 2))
        op = qtx.operator.Heisenberg(J=[1.0, 0.5], n_neighbor=[1, 2], msr=True).compiled()
        max_conn = len(op.host["f1"]) + len(op.host["f2"])
        ws = torch.empty(L.lib().qgx_resconv_eloc_workspace_bytes(Ls, ns, max_conn), dtype=torch.uint8,
                         device="cuda")
        er = torch.empty(ns, dtype=torch.float64, device="cuda")
        ei = torch.empty(ns, dtype=torch.float64, device="cuda")
        fn = lambda: L.call("qgx_resconv_eloc", L.ptr(table), Ls, B, Cc, 1, prec, C.byref(op.struct), L.ptr(spins), ns,
                            L.ptr(er), L.ptr(ei), L.ptr(ws), ws.numel(), st)
        ms = _events(fn, a.reps)
        res.update(ms=ms, samples_per_s=ns / ms * 1e3)
    else:
        O = torch.empty((2 * ns, npar), dtype=torch.float32, device="cuda")
        ws = torch.empty(L.lib().qgx_resconv_jacobian_workspace_bytes(Ls, B, Cc), dtype=torch.uint8, device="cuda")
        fn = lambda: L.call("qgx_resconv_jacobian", L.ptr(table), Ls, B, Cc, 1, L.ptr(spins), ns, L.ptr(O[:ns]),
                            L.ptr(O[ns:]), npar, L.ptr(ws), ws.numel(), st)
        ms = _events(fn, a.reps)
        res.update(ms=ms, samples_per_s=ns / ms * 1e3, o_write_gbs=2 * ns * npar * 4 / ms / 1e6)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("kernel", choices=["gram", "sweep", "eloc", "obar", "rc_forward", "rc_sweep", "rc_eloc",
                                       "rc_jacobian", "chol", "dgemm"])
    ap.add_argument("--lib", action="store_true", help="chol: cuSOLVER's FP64 Xpotrf instead of qgx_cholesky")
    ap.add_argument("--L", type=int, default=10)
    ap.add_argument("--blocks", type=int, default=8)
    ap.add_argument("--channels", type=int, default=16)
    ap.add_argument("--mode", default="tf32", choices=["fp32", "tf32", "bf16", "3xtf32"])
    ap.add_argument("--conv", default="fp32", choices=["fp32", "tf32", "bf16", "bf16_grouped"],
                    help="ResConv forward convolution arithmetic")
    ap.add_argument("--rows", type=int, default=2048)
    ap.add_argument("--k", type=int, default=16640)
    ap.add_argument("--ns", type=int, default=8192)
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--m", type=int, default=256)
    ap.add_argument("--steps", type=int, default=64)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    _build.build()
    st = L.stream_ptr()
    out = {"kernel": a.kernel}
    if a.kernel == "gram":
        A = torch.randn((a.rows, a.k), dtype=torch.float32, device="cuda") * 1e-2
        T = torch.empty((a.rows, a.rows), dtype=torch.float64, device="cuda")
        if a.mode == "bf16":
            Ab = torch.empty((a.rows, a.k), dtype=torch.bfloat16, device="cuda")
            L.call("qgx_f32_to_bf16", L.ptr(A), a.rows, a.k, a.k, L.ptr(Ab), a.k, st)
            fn = lambda: L.call("qgx_gram_tc", L.ptr(Ab), 1, a.rows, a.k, a.k, L.ptr(T), a.rows, None, st)
        else:
            mode = {"fp32": L.GRAM_FP32, "tf32": L.GRAM_TF32, "3xtf32": L.GRAM_3XTF32}[a.mode]
            fn = lambda: L.call("qgx_gram", L.ptr(A), a.rows, a.k, a.k, L.ptr(T), a.rows, mode, st)
        ms = _events(fn, a.reps)
        syrk = float(a.rows) * (a.rows + 1) * a.k
        out.update(mode=a.mode, rows=a.rows, k=a.k, ms=ms, syrk_tflops=syrk / ms / 1e9,
                   gemm_equiv_tflops=2.0 * a.rows * a.rows * a.k / ms / 1e9)
    elif a.kernel == "dgemm":
        # the FP64 pipe's rate through the library GEMM (cuBLAS DGEMM via torch.matmul), n^3 square
        n = a.rows
        X = torch.randn((n, n), dtype=torch.float64, device="cuda")
        Y = torch.randn((n, n), dtype=torch.float64, device="cuda")
        Z = torch.empty((n, n), dtype=torch.float64, device="cuda")
        ms = _events(lambda: torch.matmul(X, Y, out=Z), a.reps)
        out.update(n=n, ms=ms, fp64_tflops=2.0 * n ** 3 / ms / 1e9)
    elif a.kernel == "chol":
        # T = G G^T / k + 1e-4 I from an FP32 G of rows x k (the MinSR Gram's structure), factored
        # from a fresh copy every repetition (the copy is timed apart and subtracted)
        import ctypes as C
        n = a.rows
        G = torch.randn((n, a.k), dtype=torch.float32, device="cuda").double() / np.sqrt(a.k)
        T0 = G @ G.T + 1e-4 * torch.eye(n, dtype=torch.float64, device="cuda")
        del G
        T = torch.empty_like(T0)
        info = torch.zeros(1, dtype=torch.int32, device="cuda")
        if a.lib:
            A32 = torch.zeros((n, 8), dtype=torch.float32, device="cuda")
            b = torch.zeros(n, dtype=torch.float64, device="cuda")
            x = torch.empty(8, dtype=torch.float64, device="cuda")
            nb = C.c_int64(0)
            L.call("qgx_solve_workspace_bytes", n, 8, L.SOLVE_SHIFT_LIB, C.byref(nb))
            ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
            # the solve with zero shifts: the factorisation plus two triangular solves and a
            # projection over an 8-column A (the latter two are microseconds)
            fn = lambda: (T.copy_(T0), L.call("qgx_minsr_solve", L.ptr(T), n, L.ptr(A32), 8, 8, L.ptr(b),
                                                L.SOLVE_SHIFT_LIB, 0.0, 0.0, 0.0, 0.0, 0.0, L.ptr(x), L.ptr(info),
                                                L.ptr(ws), ws.numel(), st))
        else:
            ws = torch.empty(L.lib().qgx_cholesky_workspace_bytes(n), dtype=torch.uint8, device="cuda")
            fn = lambda: (T.copy_(T0), L.call("qgx_cholesky", L.ptr(T), n, n, L.ptr(info), None, L.ptr(ws),
                                                ws.numel(), st))
        ms = _events(fn, a.reps)
        copy_ms = _events(lambda: T.copy_(T0), a.reps)
        f = ms - copy_ms
        out.update(lib=a.lib, n=n, ms=f, copy_ms=copy_ms, info=int(info.item()),
                   fp64_tflops=n ** 3 / 3.0 / f / 1e9)
    elif a.kernel.startswith("rc_"):
        out.update(_resconv(a, st))
    else:
        table, spins = _rbm(a.n, a.m, a.ns)
        if a.kernel == "sweep":
            lp = torch.empty(a.ns, dtype=torch.float32, device="cuda")
            fn = lambda: L.call("qgx_rbm_sweep", L.ptr(table), a.n, a.m, L.ptr(spins), L.ptr(lp), None, a.ns,
                                a.steps, 7, 0, 2.0, L.PROPOSAL_LOCAL_FLIP, None, 0, 1, st)
            ms = _events(fn, a.reps)
            out.update(ns=a.ns, n=a.n, m=a.m, steps=a.steps, ms=ms,
                       proposals_per_s=a.ns * a.steps / ms * 1e3)
        elif a.kernel == "eloc":
            import quantax_gb300 as qtx
            qtx.sites.Chain(a.n)
            op = qtx.operator.Ising(h=1.0).compiled()
            import ctypes as C
            E = torch.empty(a.ns, dtype=torch.float64, device="cuda")
            fn = lambda: L.call("qgx_rbm_eloc", L.ptr(table), a.n, a.m, C.byref(op.struct), L.ptr(spins), a.ns,
                                L.ptr(E), st)
            ms = _events(fn, a.reps)
            out.update(ns=a.ns, n=a.n, m=a.m, ms=ms, samples_per_s=a.ns / ms * 1e3)
        else:
            np_ = a.m * a.n + a.m
            O = torch.empty((a.ns, np_), dtype=torch.float32, device="cuda")
            om = torch.empty(np_, dtype=torch.float64, device="cuda")
            ws = torch.empty(L.lib().qgx_rbm_obar_workspace_bytes(a.n, a.m, a.ns), dtype=torch.uint8, device="cuda")
            fn = lambda: L.call("qgx_rbm_obar", L.ptr(table), a.n, a.m, 0, L.ptr(spins), None, a.ns, L.ptr(O), np_,
                                L.ptr(om), L.ptr(ws), ws.numel(), st)
            ms = _events(fn, a.reps)
            out.update(ns=a.ns, np=np_, ms=ms, obar_write_gbs=a.ns * np_ * 4 / ms / 1e6)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
