"""The ctypes mirrors of the C ABI's structs (quantax_gb300/_lib.py) against include/qgx.h: a
small C program compiled with the host compiler prints every struct's size and every field's
offset, and the ctypes layouts must agree (a mismatch would shift the fields a batched launch
or an operator table reads)."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

STRUCTS = {
    "qgx_operator_t": ("Operator", ["c0", "n_z", "z_i", "z_J", "n_zz", "zz_ij", "zz_J", "n_f1", "f1_i", "f1_J", "n_f2",
                                    "f2_ij", "f2_J"]),
    "qgx_symm_t": ("Symm", ["perm", "weight", "nperm", "z2"]),
    "qgx_rbm_sweep_job_t": ("RbmSweepJob", ["table", "n", "m", "spins", "log_psi", "accepts", "ns", "nsteps",
                                            "proposal", "seed", "step0", "reweight", "nbr", "z", "hop"]),
    "qgx_rbm_eloc_job_t": ("RbmElocJob", ["table", "n", "m", "op", "spins", "ns", "eloc"]),
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    d = tmp_path_factory.mktemp("abi")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "qgx.h"', "int main(void) {"]
    for cname, (_, fields) in STRUCTS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in fields:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "layout"
    subprocess.run([cc, "-I", str(ROOT / "include"), "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    table = {}
    for line in out.splitlines():
        name, key, val = line.split()
        table[(name, key)] = int(val)
    return table


@pytest.mark.parametrize("cname", list(STRUCTS))
def test_ctypes_struct_matches_header(c_layout, cname):
    from quantax_gb300 import _lib
    pyname, fields = STRUCTS[cname]
    cls = getattr(_lib, pyname)
    assert C.sizeof(cls) == c_layout[(cname, "size")], cname
    for f in fields:
        assert getattr(cls, f).offset == c_layout[(cname, f)], (cname, f)


def test_batch_limit_matches_header():
    from quantax_gb300 import _lib
    text = (ROOT / "include" / "qgx.h").read_text()
    assert f"#define QGX_RBM_BATCH_MAX_JOBS {_lib.RBM_BATCH_MAX_JOBS}" in text
