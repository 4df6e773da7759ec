"""Stochastic reconfiguration / MinSR in FP64 (test infrastructure only).

Restates:
  * QNGD._Omat_to_Obar / get_Obar: Obar = (O - mean_s O) * sqrt(r / Ns)
    (quantax/optimizer/sr.py:76-88);
  * SR.get_Ebar: energy = Re mean(E r), VarE = mean(|E - Emean|^2 r),
    Ebar = (E - mean E) * sqrt(r / Ns) (quantax/optimizer/sr.py:180-195);
  * QNGD.solve: real-to-complex states stack [Re; Im] (quantax/optimizer/sr.py:90-113);
  * the solvers of quantax/optimizer/solver.py:12-201: minnorm/lstsq shift (Cholesky),
    minnorm/lstsq pinv (eigh with the soft inverse 1/(l (1 + ((rtol max|l| + atol)/|l|)^6)))
    and the SNR truncation;
  * Variational.update: params - step, skipped when non-finite
    (quantax/state/variational.py:558-579).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla


def obar(O, r=None):
    ns = O.shape[0]
    r = np.ones(ns) if r is None else np.asarray(r)
    return (O - O.mean(axis=0, keepdims=True)) * np.sqrt(r / ns)[:, None]


def ebar(E, r=None):
    ns = E.shape[0]
    r = np.ones(ns) if r is None else np.asarray(r)
    emean = np.mean(E * r)
    var = np.mean(np.abs(E - emean) ** 2 * r).real
    eb = (E - np.mean(E)) * np.sqrt(r / ns)
    return eb, float(np.real(emean)), float(var)


def _rtol(dtype=np.float64):
    return {np.dtype(np.float64): 1e-12, np.dtype(np.float32): 1e-6}[np.dtype(dtype)]


def minnorm_shift(A, b, rshift=None, ashift=1e-4):
    T = A @ A.conj().T
    tr = np.trace(T).real
    shift = (_rtol() if rshift is None else rshift) * tr + ashift
    T = T + shift * np.eye(T.shape[0])
    y = sla.solve(T, b, assume_a="pos")
    return A.conj().T @ y


def lstsq_shift(A, b, rshift=None, ashift=1e-4):
    S = A.conj().T @ A
    F = A.conj().T @ b
    tr = np.trace(S).real
    shift = (_rtol() if rshift is None else rshift) * tr + ashift
    S = S + shift * np.eye(S.shape[0])
    return sla.solve(S, F, assume_a="pos")


def eigs_inv(vals, rtol=None, atol=0.0):
    a = np.abs(vals)
    rtol = _rtol() if rtol is None else rtol
    with np.errstate(divide="ignore", invalid="ignore"):
        f = 1.0 + ((rtol * a.max() + atol) / a) ** 6
        inv = 1.0 / (vals * f)
    return np.where(a > 0.0, inv, 0.0)


def sum_without_noise(inputs, tol_snr):
    x = inputs.sum(axis=0)
    if tol_snr <= 1e-6:
        return x
    xm = x / inputs.shape[0]
    xv = np.sqrt(np.mean(np.abs(inputs - xm[None, :]) ** 2, axis=0) / inputs.shape[0])
    snr = np.abs(xm) / xv
    return x / (1.0 + (tol_snr / snr) ** 6)


def minnorm_pinv(A, b, rtol=None, atol=0.0, tol_snr=0.0):
    T = A @ A.conj().T
    lam, U = np.linalg.eigh(T)
    inv = eigs_inv(lam, rtol, atol)
    rho = sum_without_noise(U.conj() * b[:, None], tol_snr)
    return A.conj().T @ (U @ (inv * rho))


def lstsq_pinv(A, b, rtol=None, atol=0.0, tol_snr=0.0):
    S = A.conj().T @ A
    lam, V = np.linalg.eigh(S)
    inv = eigs_inv(lam, rtol, atol)
    rho_sk = (A.conj() * b[:, None]) @ V.conj()
    rho = sum_without_noise(rho_sk, tol_snr)
    return V @ (inv * rho)


def auto(A, b, kind="pinv", **kw):
    if kind == "pinv":
        return minnorm_pinv(A, b, **kw) if A.shape[0] < A.shape[1] else lstsq_pinv(A, b, **kw)
    return minnorm_shift(A, b, **kw) if A.shape[0] < A.shape[1] else lstsq_shift(A, b, **kw)


def solve(Obar, Ebar, solver, complex_out=False, imag_time=True):
    """QNGD.solve (quantax/optimizer/sr.py:90-113) for states with real parameters. Real time:
    complex-output states solve with [-Im; Re] Ebar; real ones get Ebar * 1j, whose purely
    imaginary solution casts to a zero real step."""
    if complex_out:
        A = np.concatenate([Obar.real, Obar.imag], axis=0)
        b = np.concatenate([Ebar.real, Ebar.imag]) if imag_time else np.concatenate([-Ebar.imag, Ebar.real])
    else:
        if not imag_time:
            return np.zeros(Obar.shape[1])
        A, b = np.real(Obar), np.real(Ebar)
    return solver(A, b)


def pinvh(H, b, rtol=None, atol=0.0):
    """pinvh_solve (quantax/optimizer/solver.py:104-111): U diag(soft inverse) U^H b."""
    lam, U = np.linalg.eigh(H)
    return U @ (eigs_inv(lam, rtol, atol) * (U.conj().T @ b))


def time_evol_sf(Obar, Ebar):
    """TimeEvol.get_SF one-shot form (quantax/optimizer/time_evol.py:63-68)."""
    return Obar.conj().T @ Obar, Obar.conj().T @ Ebar


def time_evol_step(S, F, complex_out=True, solver=pinvh):
    """TimeEvol.solve (quantax/optimizer/time_evol.py:113-128), real parameters."""
    if not complex_out:
        return np.zeros(S.shape[0])
    return solver(S.real, -F.imag)


def update(params, step, dtype=np.float32):
    """params (stored in `dtype`) minus step cast to `dtype`, in `dtype` arithmetic."""
    if not np.all(np.isfinite(step)):
        return params, False
    p = np.asarray(params, dtype=dtype)
    return (p - np.real(step).astype(dtype)).astype(np.float64), True


# ---- momentum variants (quantax/optimizer/sr.py:198-429), on the stacked real A and b ----
def spring_step(A, b, last, mu, solver):
    b = b - mu * (A @ last)
    step = solver(A, b) + mu * last
    return step


def march_step(A, b, last, V_state, t, mu, beta, solver, a_dtype=np.float32):
    """One MARCH solve (t already incremented); A is scaled column by column and rounded to
    a_dtype, as the device stores Obar. Returns (step, new V_state)."""
    b = b - mu * (A @ last)
    if np.allclose(V_state, 0):
        V = np.ones_like(V_state)
    else:
        V = (V_state / (1 - beta ** t)) ** 0.25 + 1e-8
    As = (A * (1.0 / V)[None, :]).astype(a_dtype).astype(np.float64)
    step = solver(As, b) / V + mu * last
    V_state = beta * V_state + (1 - beta) * np.abs(step - last) ** 2
    return step, V_state


def adamsr_step(A, b, m, v, t, mu, beta, solver, a_dtype=np.float32):
    """One AdamSR step (t already incremented). Returns (step, m, v)."""
    g = solver(A, b)
    m = mu * m + (1 - mu) * g
    v = beta * v + (1 - beta) * np.abs(g) ** 2
    mh = m / (1 - mu ** t)
    vh = v / (1 - beta ** t)
    V = vh ** 0.25 + 1e-8
    b = b - A @ mh
    As = (A * (1.0 / V)[None, :]).astype(a_dtype).astype(np.float64)
    step = solver(As, b) / V + mh
    return step, m, v


# ---- further solvers of quantax/optimizer/solver.py ---------------------------------------
def sgd(A, b):
    """sgd_solver (solver.py:297-302)."""
    return A.conj().T @ b / b.shape[0]


def lstsq_shift_direct(A, b, diag_shift):
    """The solution lstsq_shift_cg (solver.py:24-47) converges to: (S + diag_shift diag(S)) x = A^H b."""
    S = A.conj().T @ A
    return np.linalg.solve(S + diag_shift * np.diag(np.diag(S)), A.conj().T @ b)


def block_pinv(A, b, blocks, rtol=None, atol=0.0):
    """block_pinv_eig (solver.py:204-259): auto pinv per layer's columns, b / nlayers."""
    out, c0 = [], 0
    for n in blocks:
        out.append(auto(A[:, c0:c0 + n], b / len(blocks), "pinv", rtol=rtol, atol=atol))
        c0 += n
    return np.concatenate(out)


def minsr_pinv(T, b, rtol=None, atol=0.0):
    """minsr_pinv_eig (solver.py:262-294) without the SNR truncation."""
    lam, U = np.linalg.eigh(T)
    return U @ (eigs_inv(lam, rtol, atol) * (U.conj().T @ b))


def er_terms(log_psi, O, H):
    """ER.get_Ebar / get_Obar (quantax/optimizer/sr.py:485-505) over a whole basis: psi =
    exp(log psi) normalised, energy = <psi|H|psi>, Ebar = H psi - energy psi, Omat = psi O with
    NaN entries set to 0, Omean = psi^H Omat, Obar = Omat - psi Omean^T. H is any matrix with
    H @ vector (dense or scipy sparse). Returns (energy, Ebar, Obar, Omean)."""
    lp = np.asarray(log_psi)
    psi = np.exp(lp - lp.real.max())
    psi = psi / np.linalg.norm(psi)
    Hpsi = H @ psi
    energy = np.vdot(psi, Hpsi)
    Ebar = Hpsi - psi * energy
    Omat = np.asarray(O) * psi[:, None]
    Omat = np.where(np.isnan(Omat), 0, Omat)
    Omean = psi.conj() @ Omat
    return energy.real, Ebar, Omat - np.outer(psi, Omean), Omean
