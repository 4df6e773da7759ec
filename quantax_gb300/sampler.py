"""Metropolis samplers (quantax/sampler/metropolis.py:76-322, common_samplers.py:14-162).

Every chain lives in one warp of the sweep kernel; a sweep of n proposals is one
kernel launch. Draw t of chain c uses Philox4x32-10 counter (c, t, tag=1) under the
sampler's 64-bit seed, and the sampler's step counter advances by n per sweep, so a
run is reproducible from the global seed and independent of launch geometry.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional, Sequence, Union

import numpy as np
import torch

from . import _lib
from .global_defs import get_sites, get_subkeys
from .state import pack_spins, unpack_spins


@dataclass
class Samples:
    """Packed configurations, log|psi| and reweight factors (sampler/samples.py:9-74)."""
    packed: torch.Tensor                       # (ns, nw) int32 words
    log_psi: torch.Tensor                      # (ns,) float32 log|psi|
    n: int
    reweight_factor: Optional[torch.Tensor] = None   # (ns,) float64, None means all ones
    state_internal: None = None

    @property
    def nsamples(self) -> int:
        return self.packed.shape[0]

    @property
    def spins(self) -> torch.Tensor:
        """(ns, N) int8 +-1 configurations."""
        return unpack_spins(self.packed, self.n)

    @property
    def psi(self) -> torch.Tensor:
        lp = self.log_psi
        return torch.exp(lp.to(torch.complex128 if lp.is_complex() else torch.float64))

    @classmethod
    def from_spins(cls, spins, log_psi=None):
        n = get_sites().Nmodes
        packed = pack_spins(spins, n)
        lp = log_psi if log_psi is not None else torch.zeros(packed.shape[0], device=packed.device)
        return cls(packed, lp, n)


class Metropolis:
    """Metropolis-Hastings driver with one Markov chain per sample."""

    proposal = None

    def __init__(self, state, nsamples: int, reweight: float = 2.0, thermal_steps: Optional[int] = None,
                 sweep_steps: Optional[int] = None, initial_spins=None):
        self._state = state
        self._nsamples = int(nsamples)
        self._reweight = float(reweight)
        n = state.Nmodes
        self._thermal_steps = 20 * n if thermal_steps is None else int(thermal_steps)
        self._sweep_steps = 2 * n if sweep_steps is None else int(sweep_steps)
        self._seed = get_subkeys()
        self._step = 0
        self._initial_spins = initial_spins
        dev = state.params.device
        self._resconv = state.model.kind == "resconv"
        shape = (self._nsamples, 2) if self._resconv else (self._nsamples,)
        self._log_psi = torch.empty(shape, dtype=torch.float32, device=dev)
        self._accepts = torch.empty(self._nsamples, dtype=torch.int32, device=dev)
        self._nbr = torch.zeros(1, dtype=torch.int32, device=dev)
        self._z = 1
        self._hop = 1
        self._setup()
        self.reset()

    def _setup(self) -> None:
        pass

    @property
    def state(self):
        return self._state

    @property
    def nsamples(self) -> int:
        return self._nsamples

    @property
    def reweight(self) -> float:
        return self._reweight

    @property
    def Nmodes(self) -> int:
        return self._state.Nmodes

    @property
    def nflips(self) -> Optional[int]:
        return None

    @property
    def accepts(self) -> torch.Tensor:
        """Per-chain accepted proposals of the last sweep."""
        return self._accepts

    def _initial(self) -> torch.Tensor:
        n = self.Nmodes
        dev = self._log_psi.device
        if self._initial_spins is not None:
            s = np.asarray(self._initial_spins)
            if s.ndim == 1:
                s = np.tile(s, (self._nsamples, 1))
            return pack_spins(s.reshape(self._nsamples, n), n)
        packed = torch.empty((self._nsamples, (n + 31) // 32), dtype=torch.int32, device=dev)
        nparticles = self._state.sites.Nparticles
        if isinstance(nparticles, tuple):
            _lib.call("qgx_spins_init_fixed_up", _lib.ptr(packed), self._nsamples, n, nparticles[0], get_subkeys(),
                      _lib.stream_ptr())
        else:
            _lib.call("qgx_spins_init_uniform", _lib.ptr(packed), self._nsamples, n, get_subkeys(), _lib.stream_ptr())
        return packed

    def reset(self) -> None:
        """Reset the chains and thermalise them (metropolis.py:159-169)."""
        self._packed = self._initial()
        if self._thermal_steps > 0:
            self.sweep(self._thermal_steps)

    def sweep(self, nsweeps: Optional[int] = None) -> Samples:
        """nsweeps proposals per chain (metropolis.py:171-215); default sweep_steps."""
        n = self._sweep_steps if nsweeps is None else int(nsweeps)
        st = self._state
        if self._resconv:
            ws = st.workspace("sweep", st.model.sweep_workspace_bytes(self._nsamples, st.symm_dev))
            st.model.sweep(st.table, self._packed, self._log_psi, self._accepts, n, self._seed, self._step,
                           self._reweight, self.proposal, self._nbr, self._z, self._hop, ws, st.symm_dev)
            lp_real = self._log_psi[:, 0].contiguous()
            lp = torch.view_as_complex(self._log_psi.clone()) if st.is_complex else lp_real
        else:
            st.model.sweep(st.table, self._packed, self._log_psi, self._accepts, n, self._seed, self._step,
                           self._reweight, self.proposal, self._nbr, self._z, self._hop)
            lp_real = self._log_psi
            lp = self._log_psi.clone()
        self._step += n
        r = None
        if self._reweight != 2.0:
            r = torch.empty(self._nsamples, dtype=torch.float64, device=self._log_psi.device)
            _lib.call("qgx_reweight_factor", _lib.ptr(lp_real), self._nsamples, self._reweight, _lib.ptr(r),
                      _lib.stream_ptr())
        return Samples(self._packed.clone(), lp, self.Nmodes, r)


class LocalFlip(Metropolis):
    """Flip one uniformly chosen spin per proposal (common_samplers.py:14-33)."""

    proposal = _lib.PROPOSAL_LOCAL_FLIP

    @property
    def nflips(self) -> int:
        return 1


class SpinExchange(Metropolis):
    """Exchange a uniformly chosen hopping spin with a random neighbour
    (common_samplers.py:58-162)."""

    proposal = _lib.PROPOSAL_SPIN_EXCHANGE

    def __init__(self, state, nsamples: int, reweight: float = 2.0, thermal_steps: Optional[int] = None,
                 sweep_steps: Optional[int] = None, initial_spins=None,
                 n_neighbor: Union[int, Sequence[int]] = 1):
        sites = state.sites
        if isinstance(sites.Nparticles, int):
            raise ValueError("The number spin-up and spin-down particles should be specified in sites for "
                             "`SpinExchange` sampler.")
        self._n_neighbor = n_neighbor
        super().__init__(state, nsamples, reweight, thermal_steps, sweep_steps, initial_spins)

    def _setup(self) -> None:
        sites = self._state.sites
        table = sites.neighbor_table(self._n_neighbor)
        self._nbr = torch.as_tensor(table, dtype=torch.int32, device=self._log_psi.device).contiguous()
        self._z = table.shape[1]
        self._hop = 1 if 2 * sites.Nparticles[0] <= sites.Nmodes else -1

    @property
    def nflips(self) -> int:
        return 2


NeighborExchange = SpinExchange
