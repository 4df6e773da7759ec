"""Build recipe of libqgx.so: nvcc for sm_103a only, translation units compiled in
parallel, linked against the shared CUDA runtime and cuSOLVER.

    python -m quantax_gb300._build [--force] [-v]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libqgx.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", "-I", str(INCLUDE)]


def nvcc() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found: the qgx CUDA library cannot be built")


def cuda_lib_dir() -> str:
    root = Path(nvcc()).resolve().parent.parent
    for d in (root / "lib64", root / "lib", root / "targets" / "sbsa-linux" / "lib",
              root / "targets" / "x86_64-linux" / "lib"):
        if (d / "libcusolver.so").exists():
            return str(d)
    return str(root / "lib64")


def sources():
    return sorted(CSRC.glob("*.cu"))


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    srcs = sources()
    objs = [BUILD / (s.stem + ".o") for s in srcs]
    jobs = []
    for s, o in zip(srcs, objs):
        if force or _stale(o, [s] + headers):
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(s), "-o", str(o)]
            if verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append((s, cmd))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            futs = {ex.submit(subprocess.run, cmd, capture_output=True, text=True): s for s, cmd in jobs}
            errors = []
            for f in cf.as_completed(futs):
                r = f.result()
                if verbose and r.stderr:
                    sys.stderr.write(r.stderr)
                if r.returncode != 0:
                    errors.append(f"{futs[f].name}:\n{r.stderr}")
            if errors:
                raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", str(LIB), *map(str, objs),
               "-L", cuda_lib_dir(), "-lcusolver", "-Xlinker", "-rpath," + cuda_lib_dir()]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
