"""quantax_gb300: the quantax VMC inner loop (Metropolis sampling, local energies,
log-derivatives, SR / MinSR) on NVIDIA GB300 (sm_103a) through the qgx C ABI.

The public names follow the reference (quantax): sites, operator, model, state,
sampler, optimizer, set_random_seed, set_default_dtype.
"""
from . import global_defs
from .global_defs import (PARTICLE_TYPE, get_default_dtype, get_sites, get_subkeys, is_default_cpl,
                          set_default_dtype, set_random_seed)
from . import sites, nn, operator, model, state, sampler, optimizer, symmetry, utils

__all__ = ["global_defs", "sites", "operator", "model", "state", "sampler", "optimizer", "symmetry", "nn", "utils", "set_random_seed",
           "set_default_dtype", "get_default_dtype", "get_sites", "get_subkeys", "is_default_cpl", "PARTICLE_TYPE"]
