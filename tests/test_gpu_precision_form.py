"""Precision form of the J1-J2 / ResConv SR step against the FP64 oracle on one seeded
sample batch: the per-step errors of log psi, E_loc, the energy, Obar and the parameter
update, for the two tensor-core forms (TF32 convolutions + TF32 Gram, BF16 convolutions +
BF16 Gram; both with the FP32-factor + FP64-refinement solve) and for the plain FP32 path.

Workload: J1-J2 (J2 = 0.5, MSR) on the 10 x 10 square, ResConv(8 blocks, 16 channels,
complex output), 64 samples of a seeded SpinExchange chain, MinSR with diagonal shift 1e-3.
The stated bounds are in BOUNDS. The measured errors are printed (pytest -s) and written
as JSON to the file QGX_PRECISION_REPORT names, if it is set.
"""
import json
import os

import numpy as np
import pytest

from oracle import operators as oops, resconv, sr as osr

pytestmark = pytest.mark.gpu

# log psi: max |error| of Re and phase; eloc: max |error| / max |E_loc|; energy: relative;
# obar: max |error| / max |Obar|; update: relative 2-norm
BOUNDS = {
    "fp32": dict(log_psi=2e-4, eloc=2e-4, energy=1e-5, obar=1e-3, update=2e-2),
    "tf32": dict(log_psi=5e-3, eloc=5e-3, energy=1e-3, obar=1e-3, update=1e-1),
    "bf16": dict(log_psi=4e-2, eloc=4e-2, energy=5e-3, obar=1e-3, update=3e-1),
}
FORMS = {"fp32": ("fp32", "fp32", "fp64"), "tf32": ("tf32", "tf32", "mixed"), "bf16": ("bf16", "bf16", "mixed")}


@pytest.mark.parametrize("form", ["fp32", "tf32", "bf16"])
def test_precision_form_step_errors(cuda, form):
    import quantax_gb300 as qtx
    conv, gram, solve = FORMS[form]
    L, B, Cc, ns, ashift = 10, 8, 16, 64, 1e-3
    qtx.set_random_seed(11)
    qtx.set_default_dtype(np.complex128)
    try:
        qtx.sites.Square(L, Nparticles=(50, 50))
        H = qtx.operator.Heisenberg(J=[1.0, 0.5], n_neighbor=[1, 2], msr=True)
        model = qtx.model.ResConv(B, Cc, out_dtype=np.complex64, conv_precision=conv)
        state = qtx.state.Variational(model)
        sampler = qtx.sampler.SpinExchange(state, ns, thermal_steps=100, sweep_steps=100)
        opt = qtx.optimizer.SR(state, H, solver=qtx.optimizer.minnorm_shift_eig(ashift=ashift, precision=solve),
                               gram=gram)
        samples = sampler.sweep()
        step = opt.get_step(samples).cpu().numpy()
        lp = samples.log_psi.cpu().numpy().astype(np.complex128)  # sampler's log psi, complex output
        Obar_dev = opt.get_Obar(samples).cpu().numpy().astype(np.float64)
        s = samples.spins.cpu().numpy()

        onet = resconv.ResConv(state.params.cpu().numpy(), L, B, Cc, True)
        ops = oops.square_j1j2(L, 0.5, True)
        lp_ref = onet.log_psi(s)
        E_ref = oops.local_energy(s, ops, onet.log_psi)
        eb, em, _ = osr.ebar(E_ref)
        Ob = osr.obar(onet.jacobian(s))
        x_ref = osr.solve(Ob, eb, lambda A, b: osr.auto(A, b, "shift", rshift=1e-6, ashift=ashift), complex_out=True)

        E_dev = H.Oloc(state, samples).cpu().numpy()
        Ob_ref = np.concatenate([Ob.real, Ob.imag], axis=0)
        err = {
            "log_psi": float(max(np.abs(lp.real - lp_ref.real).max(),
                                 np.abs(np.angle(np.exp(1j * (lp.imag - lp_ref.imag)))).max())),
            "eloc": float(np.abs(E_dev - E_ref).max() / np.abs(E_ref).max()),
            "energy": float(abs(opt.energy - em) / abs(em)),
            "obar": float(np.abs(Obar_dev - Ob_ref).max() / np.abs(Ob_ref).max()),
            "update": float(np.linalg.norm(step - x_ref) / np.linalg.norm(x_ref)),
        }
    finally:
        qtx.set_default_dtype(np.float64)
    line = {"form": form, "conv": conv, "gram": gram, "solve": solve, "errors": err, "bounds": BOUNDS[form]}
    print(json.dumps(line))
    path = os.environ.get("QGX_PRECISION_REPORT")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(line) + "\n")
    for k, v in err.items():
        assert v <= BOUNDS[form][k], (form, k, v)
