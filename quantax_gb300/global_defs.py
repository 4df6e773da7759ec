"""Process-wide settings: default dtype, random seed stream, the global Sites object.

Mirrors quantax/global_defs.py:9-137. The reference keeps a JAX threefry key and splits
subkeys from it; here the global seed feeds a counter-based 64-bit seed sequence
(SplitMix64), and every device draw uses Philox4x32-10 keyed by such a seed.
"""
from __future__ import annotations

from enum import Enum

import numpy as np
import torch

DTYPE = np.float64
_SEED = 42
_COUNTER = 0


class PARTICLE_TYPE(Enum):
    spin = 0
    spinful_fermion = 1
    spinless_fermion = 2


def set_default_dtype(dtype) -> None:
    """float64 (real wavefunctions) or complex128 (complex wavefunctions)."""
    global DTYPE
    dt = np.dtype(dtype)
    if not (np.issubdtype(dt, np.floating) or np.issubdtype(dt, np.complexfloating)):
        raise ValueError("'dtype' should be float or complex types")
    DTYPE = dt.type


def get_default_dtype():
    return DTYPE


def get_real_dtype():
    return np.finfo(DTYPE).dtype.type


def is_default_cpl() -> bool:
    return np.issubdtype(DTYPE, np.complexfloating)


def set_random_seed(seed: int) -> None:
    """Initial random seed (default 42)."""
    global _SEED, _COUNTER
    _SEED = int(seed)
    _COUNTER = 0


def _splitmix64(x: int) -> int:
    x = (x + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return x ^ (x >> 31)


def get_subkeys(num: int | None = None):
    """Fresh 64-bit seeds from the global stream (quantax/global_defs.py:75-91)."""
    global _COUNTER
    n = 1 if num is None else int(num)
    out = []
    for _ in range(n):
        _COUNTER += 1
        out.append(_splitmix64((_SEED * 0x100000001B3 + _COUNTER) & 0xFFFFFFFFFFFFFFFF))
    return out[0] if num is None else out


_SITES = None


def get_sites():
    if _SITES is None:
        raise RuntimeError("Please define the Sites (e.g. quantax_gb300.sites.Chain(L)) first.")
    return _SITES


def get_lattice():
    from .sites import Lattice
    sites = get_sites()
    if not isinstance(sites, Lattice):
        raise RuntimeError("The sites are not a lattice.")
    return sites


def _set_sites(s) -> None:
    global _SITES
    _SITES = s


def device() -> torch.device:
    from ._lib import require_cuda
    require_cuda()
    return torch.device("cuda", torch.cuda.current_device())
