"""SR / MinSR optimiser (quantax/optimizer/sr.py:17-195) and its solvers
(quantax/optimizer/solver.py:12-201).

A solver here is a description (regularisation kind, branch and tolerances) that the
device path executes: Gram matrix on the GPU (FP32 SIMT or tensor cores), FP64 Cholesky
or FP64 eigendecomposition through cuSOLVER, projection back to parameter space.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import torch

from . import _lib
from .state import VS_TYPE

def _round8(n: int) -> int:
    return (n + 7) // 8 * 8


_GRAM_MODES = {"fp32": _lib.GRAM_FP32, "tf32": _lib.GRAM_TF32, "bf16": _lib.GRAM_BF16, "3xtf32": _lib.GRAM_3XTF32,
               "fp64": _lib.GRAM_FP64}


@dataclass(frozen=True)
class Solver:
    kind: str                 # "shift" (Cholesky) or "pinv" (eigh)
    branch: str = "auto"      # "auto", "minnorm" (T = A A^T) or "lstsq" (S = A^T A)
    rshift: Optional[float] = None
    ashift: float = 1e-4
    rtol: Optional[float] = None
    atol: float = 0.0
    tol_snr: float = 0.0
    # shift solvers: "fp64" (this library's FP64 Cholesky, tensor-core trailing updates),
    # "fp64_lib" (cuSOLVER's FP64 Cholesky) or "mixed" (FP32 Cholesky + FP64 refinement)
    precision: str = "fp64"
    diag_shift: float = 0.0   # shift_cg: relative diagonal shift
    maxiter: Optional[int] = None  # shift_cg: iteration limit (default 10 Np, as jax's cg)
    blocks: Optional[tuple] = None  # block_pinv_eig: parameter counts of the layers

    def use_minnorm(self, ns: int, np_: int) -> bool:
        if self.branch == "auto":
            return ns < np_
        return self.branch == "minnorm"


def auto_pinv_eig(rtol: Optional[float] = None, atol: float = 0.0, tol_snr: float = 0.0) -> Solver:
    """solver.py:167-201"""
    return Solver("pinv", "auto", rtol=rtol, atol=atol, tol_snr=tol_snr)


def minnorm_pinv_eig(rtol: Optional[float] = None, atol: float = 0.0, tol_snr: float = 0.0) -> Solver:
    """solver.py:128-149"""
    return Solver("pinv", "minnorm", rtol=rtol, atol=atol, tol_snr=tol_snr)


def lstsq_pinv_eig(rtol: Optional[float] = None, atol: float = 0.0, tol_snr: float = 0.0) -> Solver:
    """solver.py:152-164"""
    return Solver("pinv", "lstsq", rtol=rtol, atol=atol, tol_snr=tol_snr)


def auto_shift_eig(rshift: Optional[float] = None, ashift: float = 1e-4, precision: str = "fp64") -> Solver:
    """solver.py:80-91. precision="fp64": the FP64 Cholesky of qgx_cholesky (FP64 diagonal
    blocks, exact tensor-core trailing updates); "fp64_lib": cuSOLVER's FP64 Cholesky;
    "mixed" factors in FP32 and refines the solution in FP64 (MinSR branch), falling back to
    the FP64 factorisation when the refinement stalls."""
    if precision not in ("fp64", "fp64_lib", "mixed"):
        raise ValueError(f"precision {precision!r}: expected 'fp64', 'fp64_lib' or 'mixed'")
    return Solver("shift", "auto", rshift=rshift, ashift=ashift, precision=precision)


def minnorm_shift_eig(rshift: Optional[float] = None, ashift: float = 1e-4, precision: str = "fp64") -> Solver:
    """solver.py:50-62 (see auto_shift_eig for precision)"""
    if precision not in ("fp64", "fp64_lib", "mixed"):
        raise ValueError(f"precision {precision!r}: expected 'fp64', 'fp64_lib' or 'mixed'")
    return Solver("shift", "minnorm", rshift=rshift, ashift=ashift, precision=precision)


def lstsq_shift_eig(rshift: Optional[float] = None, ashift: float = 1e-4) -> Solver:
    """solver.py:65-77"""
    return Solver("shift", "lstsq", rshift=rshift, ashift=ashift)


def lstsq_shift_cg(diag_shift: float = 0.01, rtol: float = 1e-5, atol: float = 0.0,
                   maxiter: Optional[int] = None) -> Solver:
    """solver.py:24-47: conjugate gradients on (S + diag_shift diag(S)) x = A^T b, S = A^T A
    applied without forming it; stops when |r| <= max(rtol |A^T b|, atol) (jax's cg)."""
    return Solver("shift_cg", "lstsq", rtol=rtol, atol=atol, diag_shift=float(diag_shift), maxiter=maxiter)


def sgd_solver() -> Solver:
    """solver.py:297-302: x = A^T b / len(b)."""
    return Solver("sgd")


def block_pinv_eig(state, rtol: Optional[float] = None, atol: float = 0.0, tol_snr: float = 0.0) -> Solver:
    """solver.py:204-259: auto_pinv_eig on each layer's columns of Obar with Ebar / nlayers,
    the layers being those of the model's Sequential that hold parameters."""
    blocks = tuple(int(b) for b in state.model.param_blocks())
    if sum(blocks) != state.nparams:
        raise ValueError("the model's layer sizes do not add up to its parameter count")
    return Solver("pinv", "auto", rtol=rtol, atol=atol, tol_snr=tol_snr, blocks=blocks)


class minsr_pinv_eig:
    """solver.py:262-294: x = T^+ b for a Hermitian T (FP64 device tensors), the soft
    pseudo-inverse of the eigendecomposition. Called as solver(T, b); T is not modified."""

    def __init__(self, rtol: Optional[float] = None, atol: float = 0.0, tol_snr: float = 0.0):
        if tol_snr > 1e-6:
            raise NotImplementedError("minsr_pinv_eig: the SNR truncation needs the per-sample terms")
        self.rtol, self.atol = rtol, atol

    def __call__(self, T: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
        import ctypes as C
        n = T.shape[0]
        S = T.to(torch.float64).clone()
        f = b.to(torch.float64).contiguous()
        nbytes = C.c_int64(0)
        _lib.call("qgx_solve_workspace_bytes", n, 1, _lib.SOLVE_PINV, C.byref(nbytes))
        ws = torch.empty(max(nbytes.value, 256), dtype=torch.uint8, device=T.device)
        x = torch.empty(n, dtype=torch.float64, device=T.device)
        rtol = _OBAR_RTOL if self.rtol is None else self.rtol
        _lib.call("qgx_sym_solve", _lib.ptr(S), n, _lib.ptr(f), _lib.SOLVE_PINV, 0.0, 0.0, rtol, self.atol,
                  _lib.ptr(x), None, _lib.ptr(ws), ws.numel(), _lib.stream_ptr())
        return x


# Default relative shift / eigenvalue cut-off: solver.py:12-21 takes it from the dtype of the
# matrix it factors (1e-12 float64, 1e-6 float32). Obar is FP32 here, so T = Obar Obar^T carries
# FP32 rounding (~1e-7 ||T||) whatever its storage type: 1e-6 keeps T + shift positive definite
# as ||T|| grows during training, where 1e-12 let the Cholesky break down.
_OBAR_RTOL = 1e-6


class QNGD:
    """Quantum natural gradient descent: solve Obar theta_dot = Ebar (sr.py:17-128)."""

    def __init__(self, state, imag_time: bool = True, solver: Optional[Solver] = None, gram: str = "fp32"):
        self._state = state
        self._imag_time = imag_time
        self._solver = auto_pinv_eig() if solver is None else solver
        if gram not in _GRAM_MODES:
            raise ValueError(f"gram must be one of {sorted(_GRAM_MODES)}")
        self._gram = _GRAM_MODES[gram]
        self._Omean = None
        self._buf = {}
        self.marks = None  # optional list: solve() appends ("gram", event) after the Gram build
        self.last_solve_fallback = False
        self.solve_fallbacks = 0  # mixed solves that fell back to the FP64 factorisation

    @property
    def state(self):
        return self._state

    @property
    def vs_type(self):
        return self._state.vs_type

    def _buffer(self, name, shape, dtype):
        b = self._buf.get(name)
        if b is None or tuple(b.shape) != tuple(shape) or b.dtype != dtype:
            b = torch.empty(shape, dtype=dtype, device=self._state.params.device)
            self._buf[name] = b
        return b

    def get_Ebar(self, samples):
        raise NotImplementedError

    def get_Obar(self, samples) -> torch.Tensor:
        """Obar = (O - <O>) sqrt(r / Ns) (sr.py:79-88). Rows are padded to a multiple of 8
        elements so that the tensor-core Gram can address them with TMA (16-byte strides)."""
        np_ = self._state.nparams
        out = self._buffer("obar", (self._state.obar_rows(samples.nsamples), _round8(np_)), torch.float32)
        obar, self._Omean = self._state.obar(samples, out[:, :np_])
        return obar

    @property
    def imag_time(self) -> bool:
        return self._imag_time

    def _gram_s(self, A: torch.Tensor) -> torch.Tensor:
        """S = A^T A (np x np FP64) in the Gram mode of this optimizer."""
        ns, np_ = A.shape
        st = _lib.stream_ptr()
        S = self._buffer("gram", (np_, np_), torch.float64)
        if self._gram == _lib.GRAM_FP32:
            _lib.call("qgx_gram_t", _lib.ptr(A), ns, np_, A.stride(0), _lib.ptr(S), np_, st)
        else:
            # S = A^T A as the tensor-core Gram of A^T (rows padded for 16-byte TMA strides)
            bf16 = self._gram == _lib.GRAM_BF16
            At = self._buffer("obar_t", (np_, _round8(ns)), torch.bfloat16 if bf16 else torch.float32)
            _lib.call("qgx_transpose", _lib.ptr(A), ns, np_, A.stride(0), _lib.ptr(At), At.stride(0), int(bf16), st)
            if bf16:
                _lib.call("qgx_gram_tc", _lib.ptr(At), 1, np_, ns, At.stride(0), _lib.ptr(S), np_, None, st)
            else:
                _lib.call("qgx_gram", _lib.ptr(At), np_, ns, At.stride(0), _lib.ptr(S), np_, self._gram, st)
        self._mark("gram")
        return S

    def solve(self, Obar: torch.Tensor, Ebar: torch.Tensor) -> torch.Tensor:
        """step = solver(Obar, Ebar) in FP64 (sr.py:90-113)."""
        # real_to_complex states arrive stacked: Obar rows [Re; Im], Ebar [Re; Im] (sr.py:99-105)
        A = Obar
        b = Ebar.to(torch.float64).contiguous()
        ns, np_ = A.shape
        if not self._imag_time:
            if self.vs_type != VS_TYPE.real_to_complex:
                # Ebar * 1j makes the solution purely imaginary, and its cast to the real
                # parameters keeps the real part: zero (sr.py:98-100, 111)
                return torch.zeros(np_, dtype=torch.float64, device=A.device)
            h = ns // 2
            b = torch.cat([-b[h:], b[:h]]).contiguous()  # [-Im; Re] (sr.py:105)
        sv = self._solver
        if sv.kind == "sgd":
            return self._rmatvec(A, b) / b.shape[0]
        if sv.kind == "shift_cg":
            return self._shift_cg(A, b, sv)
        if sv.blocks is not None:
            # layer by layer, Ebar / nlayers (solver.py:251-257)
            parts, c0 = [], 0
            sub = Solver(sv.kind, sv.branch, sv.rshift, sv.ashift, sv.rtol, sv.atol, sv.tol_snr, sv.precision)
            for n_i in sv.blocks:
                blk = torch.zeros((ns, _round8(n_i)), dtype=torch.float32, device=A.device)
                blk[:, :n_i].copy_(A[:, c0:c0 + n_i])  # 16-byte aligned rows for the tensor-core Gram
                parts.append(self._solve_matrix(blk[:, :n_i], b / len(sv.blocks), sub))
                c0 += n_i
            return torch.cat(parts)
        return self._solve_matrix(A, b, sv)

    def _rmatvec(self, A: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
        """A^T b (FP64) by qgx_obar_rmatvec."""
        import ctypes as C
        rows, cols = A.shape
        nb = C.c_int64(0)
        _lib.call("qgx_obar_rmatvec_workspace_bytes", rows, cols, C.byref(nb))
        ws = self._state.workspace("rmatvec", nb.value)
        y = torch.empty(cols, dtype=torch.float64, device=A.device)
        _lib.call("qgx_obar_rmatvec", _lib.ptr(A), rows, cols, A.stride(0), _lib.ptr(b), _lib.ptr(y), _lib.ptr(ws),
                  ws.numel(), _lib.stream_ptr())
        return y

    def _matvec(self, A: torch.Tensor, x: torch.Tensor) -> torch.Tensor:
        rows, cols = A.shape
        x = x.contiguous()
        y = torch.empty(rows, dtype=torch.float64, device=A.device)
        _lib.call("qgx_obar_matvec", _lib.ptr(A), rows, cols, A.stride(0), _lib.ptr(x), _lib.ptr(y),
                  _lib.stream_ptr())
        return y

    def _shift_cg(self, A: torch.Tensor, b: torch.Tensor, sv: Solver) -> torch.Tensor:
        """lstsq_shift_cg (solver.py:24-47): CG on (S + diag_shift diag(S)) x = A^T b, the Obar
        passes on the device; stops when |r| <= max(rtol |F|, atol) or after maxiter (10 Np)."""
        rows, cols = A.shape
        F = self._rmatvec(A, b)
        d = torch.empty(cols, dtype=torch.float64, device=A.device)
        ws = self._state.workspace("sumsq", int(_lib.lib().qgx_column_sumsq_workspace_bytes(rows, cols)))
        _lib.call("qgx_column_sumsq", _lib.ptr(A), rows, cols, A.stride(0), _lib.ptr(d), _lib.ptr(ws), ws.numel(),
                  _lib.stream_ptr())
        d *= sv.diag_shift
        x = torch.zeros_like(F)
        r = F.clone()
        p = r.clone()
        rs = float(r @ r)
        tol2 = max(sv.rtol * float(torch.linalg.vector_norm(F)), sv.atol) ** 2
        for _ in range(10 * cols if sv.maxiter is None else int(sv.maxiter)):
            if rs <= tol2:
                break
            Ap = self._rmatvec(A, self._matvec(A, p)) + d * p
            alpha = rs / float(p @ Ap)
            x += alpha * p
            r -= alpha * Ap
            rs_new = float(r @ r)
            p = r + (rs_new / rs) * p
            rs = rs_new
        return x

    def _solve_matrix(self, A: torch.Tensor, b: torch.Tensor, sv: Solver) -> torch.Tensor:
        """The pinv / shift solvers on the real matrix A and right-hand side b."""
        ns, np_ = A.shape
        method = _lib.SOLVE_PINV
        if sv.kind == "shift":
            method = _lib.SOLVE_SHIFT_LIB if sv.precision == "fp64_lib" else _lib.SOLVE_SHIFT
        rshift = _OBAR_RTOL if sv.rshift is None else sv.rshift
        rtol = _OBAR_RTOL if sv.rtol is None else sv.rtol
        x = torch.empty(np_, dtype=torch.float64, device=A.device)
        info = self._buffer("info", (1,), torch.int32)
        st = _lib.stream_ptr()
        L = _lib.lib()
        import ctypes as C
        nbytes = C.c_int64(0)
        if sv.use_minnorm(ns, np_):
            T = self._buffer("gram", (ns, ns), torch.float64)
            if self._gram == _lib.GRAM_BF16:
                Ab = self._buffer("obar_bf16", (ns, _round8(np_)), torch.bfloat16)
                _lib.call("qgx_f32_to_bf16", _lib.ptr(A), ns, np_, A.stride(0), _lib.ptr(Ab), Ab.stride(0), st)
                _lib.call("qgx_gram_tc", _lib.ptr(Ab), 1, ns, np_, Ab.stride(0), _lib.ptr(T), ns, None, st)
            else:
                _lib.call("qgx_gram", _lib.ptr(A), ns, np_, A.stride(0), _lib.ptr(T), ns, self._gram, st)
            self._mark("gram")
            if sv.kind == "shift" and sv.precision == "mixed":
                method = _lib.SOLVE_SHIFT_MIXED
            _lib.call("qgx_solve_workspace_bytes", ns, np_, method, C.byref(nbytes))
            ws = self._state.workspace("solve", nbytes.value)
            _lib.call("qgx_minsr_solve", _lib.ptr(T), ns, _lib.ptr(A), np_, A.stride(0), _lib.ptr(b), method, rshift,
                      sv.ashift, rtol, sv.atol, sv.tol_snr, _lib.ptr(x), _lib.ptr(info), _lib.ptr(ws), ws.numel(), st)
            if method == _lib.SOLVE_SHIFT_MIXED:
                code = int(info.item())
                self.last_solve_fallback = code != 0
                if code != 0:
                    # the FP32 factor broke down (code > 0: pivot `code` not positive) or the
                    # refinement stalled (code < 0): factor the already shifted FP64 matrix
                    self.solve_fallbacks += 1
                    _lib.call("qgx_solve_workspace_bytes", ns, np_, _lib.SOLVE_SHIFT, C.byref(nbytes))
                    ws = self._state.workspace("solve", nbytes.value)
                    # a failure here makes x NaN (the reference's Cholesky solve does the same),
                    # and Variational.update skips the step with a warning
                    _lib.call("qgx_minsr_solve", _lib.ptr(T), ns, _lib.ptr(A), np_, A.stride(0), _lib.ptr(b),
                              _lib.SOLVE_SHIFT, 0.0, 0.0, rtol, sv.atol, sv.tol_snr, _lib.ptr(x), _lib.ptr(info),
                              _lib.ptr(ws), ws.numel(), st)
        else:
            S = self._gram_s(A)
            _lib.call("qgx_solve_workspace_bytes", np_, ns, method, C.byref(nbytes))
            ws = self._state.workspace("solve", nbytes.value)
            _lib.call("qgx_sr_solve", _lib.ptr(S), np_, _lib.ptr(A), ns, A.stride(0), _lib.ptr(b), method, rshift,
                      sv.ashift, rtol, sv.atol, sv.tol_snr, _lib.ptr(x), _lib.ptr(info), _lib.ptr(ws), ws.numel(), st)
        return x

    def _mark(self, name: str) -> None:
        if self.marks is not None:
            ev = torch.cuda.Event(enable_timing=True)
            ev.record()
            self.marks.append((name, ev))

    def get_step(self, samples, local_energies: Optional[torch.Tensor] = None) -> torch.Tensor:
        """local_energies: the samples' E_loc when already computed (a batched evaluation)."""
        Ebar = self.get_Ebar(samples) if local_energies is None else self.get_Ebar(samples, local_energies)
        Obar = self.get_Obar(samples)
        return self.solve(Obar, Ebar)


class SR(QNGD):
    """Stochastic reconfiguration; MinSR when Ns < Np (sr.py:131-195)."""

    def __init__(self, state, hamiltonian, imag_time: bool = True, solver: Optional[Solver] = None,
                 gram: str = "fp32"):
        super().__init__(state, imag_time, solver, gram)
        self._hamiltonian = hamiltonian
        self._stats = None

    @property
    def hamiltonian(self):
        return self._hamiltonian

    @property
    def energy(self) -> Optional[float]:
        return None if self._stats is None else float(self._stats[0])

    @property
    def VarE(self) -> Optional[float]:
        return None if self._stats is None else float(self._stats[2])

    @property
    def stats(self) -> Optional[torch.Tensor]:
        """Device tensor [Re energy, Im energy, VarE] of the last step (no sync)."""
        return self._stats

    def get_Ebar(self, samples, local_energies: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Ebar = (E - <E>) sqrt(r / Ns); energy and VarE kept on the device (sr.py:180-195).
        local_energies: E_loc of the samples when already computed."""
        E = self._hamiltonian.Oloc(self._state, samples) if local_energies is None else local_energies
        ns = samples.nsamples
        stats = self._buffer("stats", (3,), torch.float64)
        cplx = E.is_complex()
        ebar = torch.empty(2 * ns if cplx else ns, dtype=torch.float64, device=E.device)
        er = E.real.contiguous() if cplx else E
        ei = E.imag.contiguous() if cplx else None
        _lib.call("qgx_energy_stats", _lib.ptr(er), _lib.ptr(ei), _lib.ptr(samples.reweight_factor), ns,
                  _lib.ptr(stats), _lib.ptr(ebar[:ns]), _lib.ptr(ebar[ns:]) if cplx else None, _lib.stream_ptr())
        self._stats = stats
        if cplx and self.vs_type != VS_TYPE.real_to_complex:
            raise ValueError("complex local energies need a complex-output state")
        return ebar


class _MomentumSR(SR):
    """Shared pieces of the momentum variants: Obar @ x and the in-place column scaling run on
    the device (qgx_obar_matvec / qgx_scale_columns); the O(Np) bookkeeping is elementwise."""

    _saved: tuple = ()

    def __init__(self, state, hamiltonian, imag_time, solver, gram, file):
        super().__init__(state, hamiltonian, imag_time, solver, gram)
        self._dev = state.params.device
        if file is not None:
            self.load(file)

    def _zeros(self):
        return torch.zeros(self._state.nparams, dtype=torch.float64, device=self._dev)

    def _obar_dot(self, Obar: torch.Tensor, x: torch.Tensor) -> torch.Tensor:
        rows, np_ = Obar.shape
        x = x.contiguous()
        y = torch.empty(rows, dtype=torch.float64, device=Obar.device)
        _lib.call("qgx_obar_matvec", _lib.ptr(Obar), rows, np_, Obar.stride(0), _lib.ptr(x), _lib.ptr(y),
                  _lib.stream_ptr())
        return y

    def _scale_columns(self, Obar: torch.Tensor, s: torch.Tensor) -> None:
        rows, np_ = Obar.shape
        s = s.contiguous()
        _lib.call("qgx_scale_columns", _lib.ptr(Obar), rows, np_, Obar.stride(0), _lib.ptr(s),
                  _lib.stream_ptr())

    # the momentum vectors holding steps are stored in the default dtype, as the reference's
    # solve returns them (sr.py:111); the squared ones stay real (sr.py:300-301, 382-383)
    _step_like = ("_last_step", "_m")

    def save(self, file) -> None:
        """The optimizer's internal quantities, in the reference's file format (its leaf
        order, sr.py:258-262, 344-349, 424-429): one .npy record per quantity."""
        import numpy as np
        from .checkpoint import write_leaves
        from .global_defs import is_default_cpl
        leaves = []
        for k in self._saved:
            v = getattr(self, k)
            if torch.is_tensor(v):
                v = v.cpu().numpy().astype(np.float64)
                if k in self._step_like and is_default_cpl():
                    v = v.astype(np.complex128)
            leaves.append(v)
        write_leaves(file, leaves)

    def load(self, file) -> None:
        """Quantities saved by save() or by the reference's optimizer."""
        from .checkpoint import read_leaves
        for k, v in zip(self._saved, read_leaves(file, len(self._saved))):
            if v.ndim:
                if v.shape != (self._state.nparams,):
                    raise ValueError(f"{k}: {v.shape[0]} entries in the file, the state has {self._state.nparams}")
                setattr(self, k, torch.as_tensor(v.real, dtype=torch.float64, device=self._dev))
            else:
                setattr(self, k, v.item())


class SPRING(_MomentumSR):
    """SPRING: SR with momentum (sr.py:198-262). Ebar -= mu Obar @ last_step before the solve,
    step += mu last_step after it. Obar and Ebar are the stacked real matrix / vector of
    QNGD.solve; for a real_to_complex state the correction is the same row by row."""

    _saved = ("_mu", "_last_step")

    def __init__(self, state, hamiltonian, imag_time: bool = True, solver: Optional[Solver] = None,
                 mu: float = 0.9, file=None, gram: str = "fp32"):
        self._mu = float(mu)
        self._last_step = None
        super().__init__(state, hamiltonian, imag_time, solver, gram, file)
        if self._last_step is None:
            self._last_step = self._zeros()

    def solve(self, Obar: torch.Tensor, Ebar: torch.Tensor) -> torch.Tensor:
        Ebar = Ebar.to(torch.float64) - self._mu * self._obar_dot(Obar, self._last_step)
        step = super().solve(Obar, Ebar)
        step = step + self._mu * self._last_step
        self._last_step = step
        return step


class MARCH(_MomentumSR):
    """MARCH: SR with first and second order momentum (sr.py:265-351). Obar is divided by
    V = (V_t / (1 - beta^t))^(1/4) + 1e-8 column by column, in place."""

    _saved = ("_mu", "_beta", "_last_step", "_V", "_t")

    def __init__(self, state, hamiltonian, imag_time: bool = True, solver: Optional[Solver] = None,
                 mu: float = 0.95, beta: float = 0.995, file=None, gram: str = "fp32"):
        self._mu, self._beta = float(mu), float(beta)
        self._last_step = self._V = None
        self._t = 0
        super().__init__(state, hamiltonian, imag_time, solver, gram, file)
        if self._last_step is None:
            self._last_step, self._V = self._zeros(), self._zeros()

    def solve(self, Obar: torch.Tensor, Ebar: torch.Tensor) -> torch.Tensor:
        self._t += 1
        Ebar = Ebar.to(torch.float64) - self._mu * self._obar_dot(Obar, self._last_step)
        # the reference's allclose(V, 0) test (|V| <= 1e-8 everywhere) selected on the device,
        # so the step enqueues without waiting for the device
        unset = (self._V.abs() <= 1e-8).all()
        V = torch.where(unset, torch.ones_like(self._V), (self._V / (1.0 - self._beta ** self._t)) ** 0.25 + 1e-8)
        self._scale_columns(Obar, 1.0 / V)
        step = super().solve(Obar, Ebar)
        step = step / V + self._mu * self._last_step
        self._V = self._beta * self._V + (1.0 - self._beta) * (step - self._last_step) ** 2
        self._last_step = step
        return step


class AdamSR(_MomentumSR):
    """AdamSR: two SR solves per step with Adam-style moments (sr.py:354-429)."""

    _saved = ("_mu", "_beta", "_m", "_v", "_t")

    def __init__(self, state, hamiltonian, imag_time: bool = True, solver: Optional[Solver] = None,
                 mu: float = 0.95, beta: float = 0.995, file=None, gram: str = "fp32"):
        self._mu, self._beta = float(mu), float(beta)
        self._m = self._v = None
        self._t = 0
        super().__init__(state, hamiltonian, imag_time, solver, gram, file)
        if self._m is None:
            self._m, self._v = self._zeros(), self._zeros()

    def solve(self, Obar: torch.Tensor, Ebar: torch.Tensor) -> torch.Tensor:
        self._t += 1
        Ebar = Ebar.to(torch.float64)
        g = super().solve(Obar, Ebar)
        self._m = self._mu * self._m + (1.0 - self._mu) * g
        self._v = self._beta * self._v + (1.0 - self._beta) * g ** 2
        m = self._m / (1.0 - self._mu ** self._t)
        v = self._v / (1.0 - self._beta ** self._t)
        V = v ** 0.25 + 1e-8
        Ebar = Ebar - self._obar_dot(Obar, m)
        self._scale_columns(Obar, 1.0 / V)
        step = super().solve(Obar, Ebar)
        return step / V + m


class ER(QNGD):
    """Exact reconfiguration (sr.py:432-513): Obar theta_dot = Ebar summed over a whole basis
    instead of samples, for small systems.

    The basis is the computational one of the sites' fixed-magnetisation sector (all 2^N
    configurations without Nparticles). The reference sums over the representatives of its
    symmetry's QuSpin basis with psi(rep) / norm(rep) as coefficients. A state projected on
    that symmetry lies in the span of the symmetric vectors, onto which the representatives'
    orthonormal vectors map isometrically, so Ebar, Obar^H Obar, Obar^H Ebar and the step are
    the same in either basis; the full basis costs |G| times more forwards.

    On the device: psi by the model's forward over the basis, H psi as a CSR product
    (qgx_csr_matvec), Omat = psi O by qgx_er_weight_rows after the jacobian kernel, Omean =
    psi^H Omat by qgx_obar_rmatvec, Obar = Omat - psi Omean^T by qgx_er_center, then the
    SR / MinSR solve. The Gram defaults to the FP64-class mode: an exact step has no sampling
    noise to hide FP32 Gram rounding behind."""

    def __init__(self, state, hamiltonian, imag_time: bool = True, solver: Optional[Solver] = None, symm=None,
                 gram: str = "fp64"):
        import numpy as np
        from .global_defs import get_sites
        from .state import pack_spins
        super().__init__(state, imag_time, solver, gram)
        if symm is not None and symm is not state.symm and not (symm.is_identity and state.symm.is_identity):
            raise NotImplementedError("ER sums over the sector of the state's own symmetry: pass symm=None")
        self._hamiltonian = hamiltonian
        self._energy = None
        sites = get_sites()
        nup = sites.Nparticles[0] if isinstance(sites.Nparticles, tuple) else None
        H, states = hamiltonian.to_sparse(nup, return_states=True)
        H = H.tocsr()
        H.sort_indices()
        n = state.Nmodes
        spins = (((states[:, None] >> np.arange(n)) & 1) * 2 - 1).astype(np.int8)
        dev = state.params.device
        self._spins = spins
        self._packed = pack_spins(spins, n)
        self._rowptr = torch.as_tensor(H.indptr.astype(np.int64), device=dev)
        self._col = torch.as_tensor(H.indices.astype(np.int32), device=dev)
        self._val = torch.as_tensor(H.data.astype(np.float64), device=dev)
        self._dim = len(states)

    @property
    def hamiltonian(self):
        return self._hamiltonian

    @property
    def energy(self) -> Optional[float]:
        return self._energy

    @property
    def basis_spins(self):
        """The basis configurations (dim x N, +-1 int8, numpy)."""
        return self._spins

    def psi(self) -> torch.Tensor:
        """The normalised amplitudes over the basis (float64, complex128 for complex output)."""
        lp = self._state.log_psi_packed(self._packed)
        lp = lp.to(torch.complex128 if lp.is_complex() else torch.float64)
        psi = torch.exp(lp - lp.real.max())  # the normalisation below removes the shift
        if psi.is_complex() and not self._state.is_complex:
            psi = psi.real  # a signed real state: phase 0 or pi
        return psi / torch.linalg.vector_norm(psi)

    @staticmethod
    def _pairs(psi: torch.Tensor) -> torch.Tensor:
        return (torch.view_as_real(psi) if psi.is_complex() else psi).contiguous()

    def get_Ebar(self, psi: torch.Tensor) -> torch.Tensor:
        """Ebar = H psi - <psi|H|psi> psi (sr.py:488-495); [Re; Im] stacked for complex output,
        the layout solve() takes."""
        x = self._pairs(psi)
        y = torch.empty_like(x)
        _lib.call("qgx_csr_matvec", _lib.ptr(self._rowptr), _lib.ptr(self._col), _lib.ptr(self._val), self._dim,
                  _lib.ptr(x), 2 if psi.is_complex() else 1, _lib.ptr(y), _lib.stream_ptr())
        Hpsi = torch.view_as_complex(y) if psi.is_complex() else y
        energy = torch.vdot(psi, Hpsi)
        self._energy = float(energy.real)
        ebar = Hpsi - psi * energy
        return torch.cat([ebar.real, ebar.imag]).contiguous() if ebar.is_complex() else ebar

    def get_Obar(self, psi: torch.Tensor) -> torch.Tensor:
        """Obar = psi O - psi Omean^T with Omean = psi^H (psi O) (sr.py:497-505): FP32 rows,
        [Re; Im] stacked for complex output, padded to 16-byte strides for the Gram."""
        st = self._state
        np_ = st.nparams
        rows = st.obar_rows(self._dim)
        out = self._buffer("obar", (rows, _round8(np_)), torch.float32)
        O = out[:, :np_]
        st.jacobian_rows(self._packed, O)
        cplx = psi.is_complex()
        x = self._pairs(psi)
        s = _lib.stream_ptr()
        _lib.call("qgx_er_weight_rows", _lib.ptr(O), self._dim, np_, O.stride(0), _lib.ptr(x), int(cplx), s)
        if cplx:
            # Omean = sum conj(psi) Omat: Re = Re psi . Re Omat + Im psi . Im Omat,
            # Im = Re psi . Im Omat - Im psi . Re Omat, as A^T b over the stacked rows
            b_re = torch.cat([psi.real, psi.imag]).contiguous()
            b_im = torch.cat([-psi.imag, psi.real]).contiguous()
            m = torch.stack([self._rmatvec(O, b_re), self._rmatvec(O, b_im)]).contiguous()
            self._Omean = torch.complex(m[0], m[1])
        else:
            m = self._rmatvec(O, x)
            self._Omean = m
        _lib.call("qgx_er_center", _lib.ptr(O), self._dim, np_, O.stride(0), _lib.ptr(x), int(cplx), _lib.ptr(m), s)
        return O

    def get_step(self, samples=None) -> torch.Tensor:
        """The exact step; `samples` is accepted for the drivers' calling convention and unused."""
        psi = self.psi()
        Ebar = self.get_Ebar(psi)
        Obar = self.get_Obar(psi)
        return self.solve(Obar, Ebar)


def pinvh_solve(rtol: Optional[float] = None, atol: float = 0.0) -> Solver:
    """solver.py:104-111: S x = F by eigh with the soft inverse (TimeEvol's default)."""
    return Solver("pinv", "lstsq", rtol=rtol, atol=atol)


class TimeEvol(SR):
    """Real-time evolution on the S-path (time_evol.py:26-134): S = Obar^H Obar (np x np)
    and F = Obar^H Ebar, then S x = -Im F for complex-output states.

    The reference accumulates S and F over sample chunks when the samples exceed its backward
    chunk (time_evol.py:70-111); here Obar stays resident in HBM and the Gram kernel reads it
    once, so the one-shot form is the only one. The solver acts on S itself: a "pinv" solver is
    pinvh_solve, a "shift" solver the shifted Cholesky solve of S."""

    def __init__(self, state, hamiltonian, solver: Optional[Solver] = None, gram: str = "fp32"):
        super().__init__(state, hamiltonian, imag_time=False, solver=pinvh_solve() if solver is None else solver,
                         gram=gram)

    def get_SF(self, samples):
        """(S, F): S = Re(Obar^H Obar), FP64 np x np; F = Obar^H Ebar, complex128 for a
        complex-output state (else FP64). Only Re S is formed: solve() reads nothing else for
        states with real parameters (time_evol.py:119-121)."""
        S, F = self._sf(samples)
        return S.clone(), F

    def _sf(self, samples):
        Ebar = self.get_Ebar(samples).contiguous()
        Obar = self.get_Obar(samples)
        S = self._gram_s(Obar)
        rows, np_ = Obar.shape
        import ctypes as C
        nb = C.c_int64(0)
        _lib.call("qgx_obar_rmatvec_workspace_bytes", rows, np_, C.byref(nb))
        ws = self._state.workspace("rmatvec", nb.value)

        def rmatvec(b):
            y = torch.empty(np_, dtype=torch.float64, device=Obar.device)
            _lib.call("qgx_obar_rmatvec", _lib.ptr(Obar), rows, np_, Obar.stride(0), _lib.ptr(b), _lib.ptr(y),
                      _lib.ptr(ws), ws.numel(), _lib.stream_ptr())
            return y

        if self.vs_type != VS_TYPE.real_to_complex:
            return S, rmatvec(Ebar)
        h = rows // 2
        # Obar^H Ebar with Obar = Ore + i Oim, Ebar = Ere + i Eim:
        # Re = Ore^T Ere + Oim^T Eim, Im = Ore^T Eim - Oim^T Ere
        Fre = rmatvec(Ebar)
        Fim = rmatvec(torch.cat([Ebar[h:], -Ebar[:h]]))
        return S, torch.complex(Fre, Fim)

    def solve(self, Smat: torch.Tensor, Fvec: torch.Tensor) -> torch.Tensor:
        """step = solver(S, 1j F) for real_or_holomorphic states (its real part, zero, for
        real parameters), solver(Re S, -Im F) otherwise (time_evol.py:115-128)."""
        return self._solve_sf(Smat.real.to(torch.float64).clone(), Fvec)

    def _solve_sf(self, S: torch.Tensor, Fvec: torch.Tensor) -> torch.Tensor:
        """solve() on an FP64 S that it may overwrite."""
        np_ = S.shape[0]
        if self.vs_type != VS_TYPE.real_to_complex:
            return torch.zeros(np_, dtype=torch.float64, device=S.device)
        import ctypes as C
        F = (-Fvec.imag if Fvec.is_complex() else torch.zeros_like(Fvec)).to(torch.float64).contiguous()
        sv = self._solver
        method = _lib.SOLVE_SHIFT if sv.kind == "shift" else _lib.SOLVE_PINV
        rshift = _OBAR_RTOL if sv.rshift is None else sv.rshift
        rtol = _OBAR_RTOL if sv.rtol is None else sv.rtol
        nbytes = C.c_int64(0)
        _lib.call("qgx_solve_workspace_bytes", np_, 1, method, C.byref(nbytes))
        ws = self._state.workspace("solve", nbytes.value)
        x = torch.empty(np_, dtype=torch.float64, device=S.device)
        _lib.call("qgx_sym_solve", _lib.ptr(S), np_, _lib.ptr(F), method, rshift, sv.ashift, rtol, sv.atol,
                  _lib.ptr(x), None, _lib.ptr(ws), ws.numel(), _lib.stream_ptr())
        return x

    def get_step(self, samples) -> torch.Tensor:
        r = samples.reweight_factor
        if r is not None and not bool(torch.allclose(r, torch.ones_like(r))):
            raise ValueError("TimeEvol is only for non-reweighted samples")
        S, F = self._sf(samples)
        return self._solve_sf(S, F)


MinSR = SR


# ---- time-stepping drivers (optimizer/driver.py) ---------------------------------------------
class Driver:
    """A sampler and an optimizer stepped with a step length; energy and VarE traced against
    the accumulated time (driver.py:9-27)."""

    def __init__(self, state, sampler, optimizer, step_length: float):
        from .utils import DataTracer
        self._state = state
        self._sampler = sampler
        self._optimizer = optimizer
        self._step_length = step_length
        self._time = 0.0
        self.energy = DataTracer()
        self.VarE = DataTracer()

    @property
    def time(self) -> float:
        return self._time

    @property
    def step_length(self) -> float:
        return self._step_length

    def step(self) -> None:
        """One iteration."""


class Euler(Driver):
    """First-order Euler driver (driver.py:30-39): theta -= dt * step(samples)."""

    def step(self) -> None:
        samples = self._sampler.sweep()
        step = self._optimizer.get_step(samples)
        self._state.update(self._step_length * step)
        self._time += self._step_length
        self.energy.append(self._optimizer.energy, self._time)
        self.VarE.append(self._optimizer.VarE, self._time)


class AdaptiveHeunEvolution(Driver):
    """Adaptive second-order Heun driver for unitary evolution (driver.py:42-104).

    Per call: a full Euler step and two half steps from the same start, five sweeps and
    TimeEvol solves; the error estimate sqrt(d^T S d) dt of the two results' difference d
    against the last S scales the next step length by (threshold / error)^(1/3), clipped to
    [0.2, 2] and the length to [1e-4, 1e-2]. As in the reference, the time advances by the new
    step length, and the state keeps the two-half-step result. The reference also forms the
    global-phase rates 1j E - Omean . step, used only by lines it leaves commented out; they are
    not computed here."""

    def __init__(self, state, sampler, tdvp, step_length: float = 1e-3, integ_threshold: float = 1e-3):
        from .utils import DataTracer
        super().__init__(state, sampler, tdvp, step_length)
        self._integ_threshold = integ_threshold
        self.step_size = DataTracer()

    def step(self) -> None:
        import numpy as np
        tdvp = self._optimizer
        st = self._state
        dt = self._step_length

        stepi = tdvp.get_step(self._sampler.sweep())
        st.update(dt * stepi)
        stepf = tdvp.get_step(self._sampler.sweep())
        step1 = (stepi + stepf) / 2
        st.update(-dt / 2 * stepi)

        stepm = tdvp.get_step(self._sampler.sweep())
        st.update(dt / 4 * (stepm - stepi))
        stepmm = tdvp.get_step(self._sampler.sweep())
        st.update(dt / 2 * stepmm)

        Smat, Fvec = tdvp.get_SF(self._sampler.sweep())
        stepff = tdvp.solve(Smat, Fvec)
        st.update(dt / 4 * (stepff - stepmm))
        step2 = (stepi + stepm + stepmm + stepff) / 4

        diff = (step1 - step2).to(Smat.dtype)
        err = float(torch.dot(diff, Smat @ diff)) if diff.numel() else 0.0
        with np.errstate(divide="ignore", invalid="ignore"):
            new_err = np.sqrt(np.float64(err)) * dt
            ratio = np.clip((np.float64(self._integ_threshold) / new_err) ** (1 / 3), 0.2, 2)
        new_step_length = float(np.clip(dt * ratio, 1e-4, 1e-2))
        self._time += new_step_length
        self._step_length = new_step_length

        self.step_size.append(new_step_length, self._time)
        self.energy.append(tdvp.energy, self._time)
        self.VarE.append(tdvp.VarE, self._time)
