"""Regenerate tests/golden/*.json.

reference_energies.json: exact-diagonalisation energies printed in the reference's own
notebooks, read as text (the reference is pure JAX and cannot be imported here).
oracle_small.json: seeded outputs of the oracle for small cases (Philox stream words,
initial configurations, a LocalFlip run, E_loc and O of an RBM), pinning the oracle's
restatement so that later changes to it are caught.

    python tests/golden/make_golden.py <path-to-reference-checkout>
"""
import json
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))


def reference_energies(ref: Path):
    out = {}

    def grab(nb, pattern):
        text = (ref / nb).read_text()
        lines = text.split("\n")
        for i, l in enumerate(lines, 1):
            m = re.search(pattern, l)
            if m:
                return float(m.group(1)), f"{nb}:{i}"
        raise RuntimeError(f"{pattern} not found in {nb}")

    v, src = grab("tutorials/J1J2.ipynb", r"Exact ground state energy: (-44\.\d+)")
    out["square4_heisenberg_msr_E0"] = dict(value=v, source=src, L=4, J=[1.0], n_neighbor=[1], msr=True, nup=8)
    v, src = grab("tutorials/J1J2.ipynb", r"Exact ground state energy: (-33\.\d+)")
    out["square4_j1j2_0.5_msr_E0"] = dict(value=v, source=src, L=4, J=[1.0, 0.5], n_neighbor=[1, 2], msr=True, nup=8)
    v, src = grab("tutorials/exact_diag.ipynb", r"E1 = (-42\.\d+)")
    out["square4_heisenberg_E1"] = dict(value=v, source=src, L=4, J=[1.0], n_neighbor=[1], msr=False, nup=8)
    v, src = grab("tutorials/exact_diag.ipynb", r"E0 = (-44\.\d+)\\n")
    out["square4_heisenberg_E0"] = dict(value=v, source=src, L=4, J=[1.0], n_neighbor=[1], msr=False, nup=8)
    return out


def reference_observables(ref: Path):
    """Expectation values the reference's notebooks print for exact ground states (read as
    text). samples.ipynb: Square(4) with no particle-number constraint, Ising(h=1) (state0) and
    Ising(h=3) (state1) ground states, M = sum_i sigma_z(i) / N, M2 = M @ M (:142); the cell at
    :342 prints state1 @ M2 @ state1 under the label "h=1.0" (state1 is the h=3 state, :34), :411
    prints exactM2[0] (the h=1 state), :451 the squared overlap of the two. exact_diag.ipynb: the
    4x4 Heisenberg() (no MSR) ground state in the Sz = 0 sector, C_ij = (sigma_z(i) sigma_z(j)
    + 2 sigma_p(i) sigma_m(j) + 2 sigma_m(i) sigma_p(j)) / 4 (:227-228), and the amplitude at the
    printed configuration s (:160-161; the sign of an eigenvector is arbitrary)."""
    out = {}

    def grab(nb, pattern, cast=float):
        lines = (ref / nb).read_text().split("\n")
        for i, l in enumerate(lines, 1):
            m = re.search(pattern, l)
            if m:
                return cast(m.group(1)), f"{nb}:{i}"
        raise RuntimeError(f"{pattern} not found in {nb}")

    v, src = grab("tutorials/samples.ipynb", r"Exact magnetization for h=1\.0: ([0-9.]+)")
    out["square4_ising_h3_M2"] = dict(value=v, source=src, L=4, h=3.0, J=1.0, observable="M2")
    v, src = grab("tutorials/samples.ipynb", r"Exact M2 = ([0-9.]+)")
    out["square4_ising_h1_M2"] = dict(value=v, source=src, L=4, h=1.0, J=1.0, observable="M2")
    v, src = grab("tutorials/samples.ipynb", r"Exact overlap:  ([0-9.]+)")
    out["square4_ising_overlap_h1_h3"] = dict(value=v, source=src, L=4, h=[1.0, 3.0], J=1.0,
                                              observable="|<psi(h=1)|psi(h=3)>|^2")
    v, src = grab("tutorials/exact_diag.ipynb", r"<C01> = (-?[0-9.]+)")
    out["square4_heisenberg_C01"] = dict(value=v, source=src, L=4, msr=False, nup=8, i=0, j=1, observable="C_ij")
    v, src = grab("tutorials/exact_diag.ipynb", r"<C02> = (-?[0-9.]+)")
    out["square4_heisenberg_C02"] = dict(value=v, source=src, L=4, msr=False, nup=8, i=0, j=2, observable="C_ij")
    spins, ssrc = grab("tutorials/exact_diag.ipynb", r'"s = \[([-0-9 ]+)\]',
                       cast=lambda t: [int(x) for x in t.split()])
    v, src = grab("tutorials/exact_diag.ipynb", r"<s\|psi0> = \[(-?[0-9.]+)\]")
    out["square4_heisenberg_psi0_at_s"] = dict(value=abs(v), source=f"{ssrc}, {src}", L=4, msr=False, nup=8,
                                               s=spins, printed_digits=6, observable="|<s|psi0>|")
    return out


def oracle_small():
    from oracle import metropolis, operators, philox, rbm
    out = {}
    ctr = philox.stream_counter(np.arange(4), np.arange(4), philox.TAG_PROPOSE)
    out["philox_seed123"] = philox.philox4x32_10(ctr, philox.seed_key(123)).tolist()
    out["init_uniform_8x70_seed5"] = metropolis.init_uniform(8, 70, 5).tolist()
    out["init_fixed_up_8x16_nup8_seed6"] = metropolis.init_fixed_up(8, 16, 8, 6).tolist()
    W, b, a = rbm.init_normal(8, 16, 0.1, seed=3, visible_bias=True)
    net = rbm.RBM(W, b, a)
    s0 = metropolis.init_uniform(16, 8, 11)
    s, lp, st = metropolis.sweep(net.log_psi, s0, 40, seed=9, step0=0)
    out["rbm_c1"] = dict(W=W.tolist(), b=b.tolist(), a=a.tolist(), s0=s0.tolist(), seed=9, nsteps=40,
                         spins=s.tolist(), log_psi=lp.tolist(), min_margin=st["min_margin"],
                         eloc=operators.local_energy(s, operators.chain_tfim(8), net.log_psi).real.tolist(),
                         jac_row0=net.jacobian(s[:1])[0].tolist())
    return out


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the quantax checkout>")
    ref = Path(sys.argv[1])
    (HERE / "reference_energies.json").write_text(
        json.dumps({**reference_energies(ref), **reference_observables(ref)}, indent=1) + "\n")
    (HERE / "oracle_small.json").write_text(json.dumps(oracle_small()) + "\n")
    print("wrote", HERE / "reference_energies.json", HERE / "oracle_small.json")
