"""Samplers: Metropolis (quantax/sampler/metropolis.py:76-322, common_samplers.py:14-162) and
the direct ones (quantax/sampler/sampler.py:14-145).

Every Metropolis chain lives in one warp of the sweep kernel; a sweep of n proposals is one
kernel launch. Draw t of chain c uses Philox4x32-10 counter (c, t, tag=1) under the
sampler's 64-bit seed, and the sampler's step counter advances by n per sweep, so a
run is reproducible from the global seed and independent of launch geometry.
"""
from __future__ import annotations

import ctypes as C
import warnings
from dataclasses import dataclass
from typing import List, Optional, Sequence, Union

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


def _reweight_factor(lp: torch.Tensor, reweight: float) -> Optional[torch.Tensor]:
    """r = |psi|^(2 - n) / mean (sampler.py:66-69) from log psi (real or complex); None for n = 2."""
    if reweight == 2.0:
        return None
    lp_real = (lp.real if lp.is_complex() else lp).to(torch.float32).contiguous()
    r = torch.empty(lp_real.shape[0], dtype=torch.float64, device=lp_real.device)
    _lib.call("qgx_reweight_factor", _lib.ptr(lp_real), lp_real.shape[0], float(reweight), _lib.ptr(r),
              _lib.stream_ptr())
    return r


class Sampler:
    """Base of the samplers (sampler.py:14-69): a state, samples per sweep and the reweight
    factor n of the sampled probability |psi|^n."""

    def __init__(self, state, nsamples: int, reweight: float = 2.0):
        self._state = state
        self._nsamples = int(nsamples)
        self._reweight = float(reweight)

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
    def Nsites(self) -> int:
        return self._state.Nsites

    @property
    def Nmodes(self) -> int:
        return self._state.Nmodes

    def sweep(self) -> "Samples":
        raise NotImplementedError


class RandomSampler(Sampler):
    """Uniformly random configurations (sampler.py:122-145): the sites' fixed-magnetisation
    sector when Nparticles is set, else all of them; reweight 0, so r = |psi|^2 / mean. Each
    sweep takes a fresh seed from the global stream, as rand_states does."""

    def __init__(self, state, nsamples: int):
        super().__init__(state, nsamples, reweight=0.0)

    def sweep(self) -> "Samples":
        n = self.Nmodes
        packed = torch.empty((self._nsamples, (n + 31) // 32), dtype=torch.int32, device=self._state.params.device)
        nparticles = self._state.sites.Nparticles
        if isinstance(nparticles, tuple):
            _lib.call("qgx_spins_init_fixed_up", _lib.ptr(packed), self._nsamples, n, nparticles[0], get_subkeys(),
                      _lib.stream_ptr())
        else:
            _lib.call("qgx_spins_init_uniform", _lib.ptr(packed), self._nsamples, n, get_subkeys(), _lib.stream_ptr())
        lp = self._state.log_psi_packed(packed)
        return Samples(packed, lp, n, _reweight_factor(lp, self._reweight))


class ExactSampler(Sampler):
    """Samples drawn directly from |psi|^n over the whole basis (sampler.py:72-119).

    The basis is every configuration of the sites' fixed-magnetisation sector (all 2^N without
    Nparticles); psi comes from the model's forward over it, once per sweep. The reference
    draws representatives of its symmetry's reduced basis with probability |<r|psi>|^n and then
    a uniform group image of each: for n = 2, or without a symmetry, that is the distribution
    |psi(s)|^n drawn here; for n != 2 with a symmetry the reference's configurations carry an
    extra factor |orbit|^(n/2 - 1) that its reweighting does not undo, and this sampler does
    not reproduce it. Sample i of sweep t is the inverse-CDF image of the 53-bit uniform of
    Philox draw (seed, i, t, tag 4) (qgx_exact_draw)."""

    def __init__(self, state, nsamples: int, reweight: float = 2.0, symm=None):
        from .utils import basis_states, states_to_spins
        super().__init__(state, nsamples, reweight)
        if symm is not None and symm is not state.symm and not (symm.is_identity and state.symm.is_identity):
            raise NotImplementedError("ExactSampler sums over the sector of the state's own symmetry: pass symm=None")
        n = self.Nmodes
        nparticles = state.sites.Nparticles
        self._states = basis_states(n, nparticles[0] if isinstance(nparticles, tuple) else None)
        self._basis = pack_spins(states_to_spins(self._states, n), n)
        self._seed = get_subkeys()
        self._step = 0
        self._last_cdf = None

    @property
    def basis_states(self) -> np.ndarray:
        """Codes of the basis configurations (bit i set = site i up)."""
        return self._states

    def probabilities(self):
        """(p, log psi): |psi|^n over the basis normalised to sum 1 (float64), and the log psi
        values it came from."""
        lp = self._state.log_psi_packed(self._basis)
        x = self._reweight * (lp.real if lp.is_complex() else lp).to(torch.float64)
        p = torch.exp(x - x[torch.isfinite(x)].max())
        p = torch.where(torch.isfinite(p) & (p > 0), p, torch.zeros_like(p))
        return p / p.sum(), lp

    def sweep(self) -> "Samples":
        p, lp = self.probabilities()
        cdf = torch.cumsum(p, 0)
        idx = torch.empty(self._nsamples, dtype=torch.int64, device=cdf.device)
        _lib.call("qgx_exact_draw", _lib.ptr(cdf), cdf.shape[0], self._nsamples, self._seed, self._step, _lib.ptr(idx),
                  _lib.stream_ptr())
        self._step += 1
        self._last_cdf = cdf
        lp_s = lp.index_select(0, idx)
        return Samples(self._basis.index_select(0, idx), lp_s, self.Nmodes, _reweight_factor(lp_s, self._reweight))


class Metropolis(Sampler):
    """Metropolis-Hastings driver with one Markov chain per sample."""

    proposal = None

    def __init__(self, state, nsamples: int, reweight: float = 2.0, thermal_steps: Optional[int] = None,
                 sweep_steps: Optional[int] = None, initial_spins=None):
        super().__init__(state, nsamples, reweight)
        n = state.Nmodes
        self._thermal_steps = 20 * n if thermal_steps is None else int(thermal_steps)
        self._sweep_steps = 2 * n if sweep_steps is None else int(sweep_steps)
        self._seed = get_subkeys()
        self._step = 0
        self._initial_spins = initial_spins
        dev = state.params.device
        # log psi as (re, im) pairs, the sweep through the batched-forward pipeline: ResConv
        # states and projected ones
        self._resconv = state.model.kind == "resconv" or state.symm_dev is not None
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

    def _device_sweep(self, nsteps: int, step0: int, proposal, nbr, z: int, hop: int) -> None:
        """nsteps proposals of one kind for every chain, Philox steps step0 .. step0 + nsteps - 1."""
        st = self._state
        if self._resconv and st.model.kind == "rbm":
            ws = st.workspace("sweep", st.model.sweep_symm_workspace_bytes(self._nsamples, st.symm_dev))
            st.model.sweep_symm(st.table, self._packed, self._log_psi, self._accepts, nsteps, self._seed, step0,
                                self._reweight, proposal, nbr, z, hop, ws, st.symm_dev)
        elif self._resconv:
            ws = st.workspace("sweep", st.model.sweep_workspace_bytes(self._nsamples, st.symm_dev))
            st.model.sweep(st.table, self._packed, self._log_psi, self._accepts, nsteps, self._seed, step0,
                           self._reweight, proposal, nbr, z, hop, ws, st.symm_dev)
        else:
            st.model.sweep(st.table, self._packed, self._log_psi, self._accepts, nsteps, self._seed, step0,
                           self._reweight, proposal, nbr, z, hop)

    def _check_local_updates(self) -> None:
        """metropolis.py:201-213: after a sweep by local updates, log|psi| is evaluated again by a
        direct forward and the direct values replace the local ones; the number of samples that
        differ (neither |psi_l - psi_d| < 1e-8 nor |psi_l / psi_d - 1| < 1e-3) is copied to the
        host without stalling it and reported by a warning when it is read: at the start of the
        next sweep, or by check_local_updates()."""
        direct = self._state.log_psi_packed(self._packed)
        if not hasattr(self, "_mismatch"):
            self._mismatch = torch.zeros(1, dtype=torch.int32, device=self._log_psi.device)
            self._mismatch_host = torch.zeros(1, dtype=torch.int32).pin_memory()
        self.check_local_updates()  # a previous count still in flight is read first
        _lib.call("qgx_log_psi_mismatch", _lib.ptr(self._log_psi), _lib.ptr(direct), self._nsamples,
                  _lib.ptr(self._mismatch), _lib.ptr(self._log_psi), _lib.stream_ptr())
        self._mismatch_host.copy_(self._mismatch, non_blocking=True)
        self._mismatch_event = torch.cuda.Event()
        self._mismatch_event.record()

    def check_local_updates(self) -> int:
        """Wait for the last sweep's psi check and warn if samples differed; returns their number
        (0 when no check is pending)."""
        ev = getattr(self, "_mismatch_event", None)
        if ev is None:
            return 0
        ev.synchronize()
        self._mismatch_event = None
        ndiff = int(self._mismatch_host[0])
        if ndiff > 0:
            warnings.warn(f"{ndiff} out of {self._nsamples} wavefunctions are not close in direct forward pass and "
                          "local updates. This may indicate inaccurate local updates.")
        return ndiff

    def _run_proposals(self, n: int) -> None:
        self._device_sweep(n, self._step, self.proposal, self._nbr, self._z, self._hop)

    def sweep(self, nsweeps: Optional[int] = None) -> Samples:
        """nsweeps proposals per chain (metropolis.py:171-215); default sweep_steps."""
        n = self._sweep_steps if nsweeps is None else int(nsweeps)
        self._run_proposals(n)
        return self._finish_sweep(n)

    def _batch_job(self, n: int):
        """The qgx_rbm_sweep_job_t of this sampler's next n proposals, or None when the sweep
        cannot join a batched launch (ResConv states, mixtures of proposal kinds)."""
        if self._resconv or type(self)._run_proposals is not Metropolis._run_proposals or self.proposal is None:
            return None
        st = self._state
        m = st.model
        return _lib.RbmSweepJob(_lib.ptr(st.table), m.N, m.M, _lib.ptr(self._packed), _lib.ptr(self._log_psi),
                                _lib.ptr(self._accepts), self._nsamples, int(n), int(self.proposal), int(self._seed),
                                int(self._step), float(self._reweight), _lib.ptr(self._nbr), int(self._z),
                                int(self._hop))

    @staticmethod
    def sweep_batched(samplers: Sequence["Metropolis"], nsweeps: Optional[int] = None) -> List[Samples]:
        """sweep() of several independent RBM samplers with their Metropolis steps in as few
        kernel launches as their shapes allow (qgx_rbm_sweep_batched: one per hidden-unit width
        class); each sampler's chains, log psi and accept counts are bit for bit those of its own
        sweep(). Samplers that cannot join a batch (ResConv, MixSampler) sweep on their own."""
        ns = [smp._sweep_steps if nsweeps is None else int(nsweeps) for smp in samplers]
        jobs, members = [], []
        for smp, n in zip(samplers, ns):
            job = smp._batch_job(n)
            if job is None:
                smp._run_proposals(n)
            else:
                jobs.append(job)
                members.append(smp)
        for i in range(0, len(jobs), _lib.RBM_BATCH_MAX_JOBS):
            chunk = jobs[i:i + _lib.RBM_BATCH_MAX_JOBS]
            arr = (_lib.RbmSweepJob * len(chunk))(*chunk)
            launches = C.c_int32(0)
            _lib.call("qgx_rbm_sweep_batched", arr, len(chunk), C.byref(launches), _lib.stream_ptr())
        return [smp._finish_sweep(n) for smp, n in zip(samplers, ns)]

    def _finish_sweep(self, n: int) -> Samples:
        """The bookkeeping after n proposals: the psi check of local updates, the step counter,
        the reweighting factors and the Samples."""
        st = self._state
        if self._resconv:
            lp_real = self._log_psi[:, 0].contiguous()
            # complex output, or a real state that can be negative (symmetry projection,
            # sinhp1): the phase carries the sign
            signed = st.symm_dev is not None or getattr(st.model, "signed_output", False)
            lp = torch.view_as_complex(self._log_psi.clone()) if st.is_complex or signed else lp_real
        else:
            if st.use_ref and self.nflips is not None:
                self._check_local_updates()
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


class MixSampler(Metropolis):
    """A mixture of Metropolis samplers (metropolis.py:325-428): every proposal step draws one
    component with probability proportional to its nsamples, and all chains propose with that
    component's move. The chains start from the components' chains, concatenated.

    Components are the built-in samplers (LocalFlip, SpinExchange with any n_neighbor); their
    moves run inside the device sweep kernels, so a Python-level propose() cannot take part.
    The component index of each step comes from a host generator seeded by (seed, step); a run
    of equal indices is one kernel sweep."""

    def __init__(self, samplers: Sequence[Metropolis], reweight: float = 2.0, thermal_steps: Optional[int] = None,
                 sweep_steps: Optional[int] = None, initial_spins=None):
        samplers = tuple(samplers)
        state = samplers[0].state
        for smp in samplers[1:]:
            if smp.state is not state:
                raise ValueError("The states of component samplers should be the same in `MixSampler`.")
        for smp in samplers:
            if type(smp).proposal is None:
                raise NotImplementedError(f"{type(smp).__name__}: only built-in proposals run in the device sweep")
            if state.model.kind == "resconv" and smp.proposal != _lib.PROPOSAL_SPIN_EXCHANGE:
                raise NotImplementedError("the ResConv sweep implements SpinExchange proposals")
        self._samplers = samplers
        counts = np.array([smp.nsamples for smp in samplers], dtype=np.float64)
        self._ratio = counts / counts.sum()
        super().__init__(state, int(counts.sum()), reweight, thermal_steps, sweep_steps, initial_spins)

    @property
    def samplers(self):
        return self._samplers

    @property
    def nflips(self) -> Optional[int]:
        nf = [smp.nflips for smp in self._samplers]
        return None if None in nf else max(nf)

    def _initial(self) -> torch.Tensor:
        if self._initial_spins is not None:
            return super()._initial()
        return torch.cat([smp._packed for smp in self._samplers], dim=0)

    def component_sequence(self, n: int, step0: int) -> np.ndarray:
        """The component drawn at each of the steps step0 .. step0 + n - 1."""
        rng = np.random.default_rng([int(self._seed), int(step0)])
        return rng.choice(len(self._samplers), size=n, p=self._ratio)

    def _run_proposals(self, n: int) -> None:
        idx = self.component_sequence(n, self._step)
        total = torch.zeros_like(self._accepts)  # each kernel sweep restarts the per-chain counts
        i = 0
        while i < n:
            j = i
            while j < n and idx[j] == idx[i]:
                j += 1
            c = self._samplers[idx[i]]
            self._device_sweep(j - i, self._step + i, c.proposal, c._nbr, c._z, c._hop)
            total += self._accepts
            i = j
        self._accepts.copy_(total)
