"""Variational state: device-resident parameters and the model kernels behind the
reference's State protocol (quantax/state/variational.py:97-587).
"""
from __future__ import annotations

import warnings
from enum import Enum
from typing import Optional

import numpy as np
import torch

from . import _lib
from .global_defs import device, get_sites, is_default_cpl


class VS_TYPE(Enum):
    """quantax/state/variational.py:40-94"""
    real_or_holomorphic = 0
    non_holomorphic = 1
    real_to_complex = 2


def _words(n: int) -> int:
    return (n + 31) // 32


def pack_spins(spins, n: Optional[int] = None) -> torch.Tensor:
    """+-1 configurations (numpy or torch, (ns, N)) -> packed int32 words on the device."""
    dev = device()
    s = torch.as_tensor(np.asarray(spins) if not isinstance(spins, torch.Tensor) else spins)
    s = s.reshape(-1, s.shape[-1] if n is None else n).to(device=dev, dtype=torch.int8).contiguous()
    ns, n = s.shape
    out = torch.empty((ns, _words(n)), dtype=torch.int32, device=dev)
    _lib.call("qgx_spins_pack", _lib.ptr(s), _lib.ptr(out), ns, n, _lib.stream_ptr())
    return out


def unpack_spins(packed: torch.Tensor, n: int) -> torch.Tensor:
    out = torch.empty((packed.shape[0], n), dtype=torch.int8, device=packed.device)
    _lib.call("qgx_spins_unpack", _lib.ptr(packed), _lib.ptr(out), packed.shape[0], n, _lib.stream_ptr())
    return out


class Variational:
    """Variational state wrapping a model with device kernels."""

    def __init__(self, model, param_file=None, symm=None, max_parallel=None, use_ref: bool = True):
        from .symmetry import Identity
        self._symm = Identity() if symm is None else symm
        if self._symm.Nmodes != get_sites().Nmodes:
            raise ValueError("the symmetry was built for another lattice")
        self._sym = None if self._symm.is_identity else self._symm
        if self._sym is not None and getattr(model, "conv", False):
            raise NotImplementedError("symmetry projection is built for ResConv and RBM_Dense")
        self._model = model
        self._dev = device()
        self._sites = get_sites()  # the lattice this state was built on (kept, not re-read)
        params = model.init_params
        if param_file is not None:
            # the reference's checkpoint (equinox leaf records) or a flat .npy of the parameters
            from .checkpoint import load_model
            params = load_model(param_file, model)
        self._params = torch.as_tensor(params, dtype=torch.float32, device=self._dev).contiguous()
        self._table = torch.empty(max(model.table_floats(), 4), dtype=torch.float32, device=self._dev)
        self._flag = torch.zeros(1, dtype=torch.int32, device=self._dev)
        self._flag_host = torch.zeros(1, dtype=torch.int32).pin_memory()
        self._flag_event = None
        self._use_ref = use_ref
        if getattr(model, "complex_output", False) and not is_default_cpl():
            raise ValueError("a complex-output model needs set_default_dtype(np.complex128) (VS_TYPE real_to_complex)")
        # a projected RBM with complex characters has a complex psi_symm: its O rows are [Re; Im]
        # when the computation dtype is complex (VS_TYPE real_to_complex, variational.py:245-255)
        self._rbm_symm_cpl = (self._sym is not None and model.kind == "rbm" and is_default_cpl()
                              and bool(np.any(np.imag(self._symm.weights()) != 0)))
        is_cpl = is_default_cpl() and getattr(model, "complex_output", False) or self._rbm_symm_cpl
        self._vs_type = VS_TYPE.real_to_complex if is_cpl else VS_TYPE.real_or_holomorphic
        self._ws = {}
        self._refresh()

    # ---- properties ----------------------------------------------------------------------
    @property
    def model(self):
        return self._model

    @property
    def nparams(self) -> int:
        return self._model.nparams

    @property
    def sites(self):
        return self._sites

    @property
    def Nsites(self) -> int:
        return self._sites.Nsites

    @property
    def Nmodes(self) -> int:
        return self._sites.Nmodes

    @property
    def vs_type(self) -> VS_TYPE:
        return self._vs_type

    @property
    def symm(self):
        """The symmetry the wavefunction is projected on (Identity by default)."""
        return self._symm

    @property
    def symm_dev(self):
        """The symmetry the kernels evaluate: None for the identity."""
        return self._sym

    @property
    def use_ref(self) -> bool:
        return self._use_ref

    @property
    def params(self) -> torch.Tensor:
        """Flat float32 parameters on the device (reference ravel order)."""
        return self._params

    @property
    def table(self) -> torch.Tensor:
        return self._table

    def _refresh(self) -> None:
        self._model.prepare(self._params, self._table)

    def workspace(self, name: str, nbytes: int) -> torch.Tensor:
        """Cached uint8 device buffer of at least nbytes (256-byte aligned by the allocator)."""
        buf = self._ws.get(name)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=self._dev)
            self._ws[name] = buf
        return buf

    # ---- forward ------------------------------------------------------------------------
    @property
    def is_complex(self) -> bool:
        return bool(getattr(self._model, "complex_output", False)) or self._rbm_symm_cpl

    def log_psi_packed(self, packed: torch.Tensor) -> torch.Tensor:
        """log psi of packed configurations: float32, or complex64 for complex-output models."""
        if self._model.kind == "rbm" and self._sym is None:
            out = torch.empty(packed.shape[0], dtype=torch.float32, device=self._dev)
            self._model.log_psi(self._table, packed, out)
            return out
        out = torch.empty((packed.shape[0], 2), dtype=torch.float32, device=self._dev)
        if self._model.kind == "rbm":
            ws = self.workspace("fwd_symm", self._model.log_psi_symm_workspace_bytes(packed.shape[0], self._sym))
            self._model.log_psi_symm(self._table, packed, out, self._sym, ws)
        elif self._sym is None:
            self._model.log_psi(self._table, packed, out)
        else:
            ws = self.workspace("fwd_symm", self._model.log_psi_workspace_bytes(packed.shape[0], self._sym))
            self._model.log_psi(self._table, packed, out, self._sym, ws)
        # a projected or sinhp1 real state can be negative: its phase (0 or pi) carries the sign
        if self.is_complex or self._sym is not None or getattr(self._model, "signed_output", False):
            return torch.view_as_complex(out)
        return out[:, 0].contiguous()

    def log_psi(self, s) -> torch.Tensor:
        return self.log_psi_packed(pack_spins(s, self.Nmodes))

    def __call__(self, s) -> torch.Tensor:
        """psi(s) as float64 / complex128 (variational.py:325-347); use log_psi for large systems."""
        lp = self.log_psi(s)
        psi = torch.exp(lp.to(torch.complex128 if lp.is_complex() else torch.float64))
        return psi if self.is_complex or not psi.is_complex() else psi.real

    def init_internal(self, s):
        return None

    # ---- local energies and log-derivatives ---------------------------------------------
    def local_energy(self, op, samples) -> torch.Tensor:
        """E_loc per sample: float64, or complex128 for complex-output models."""
        comp = op.compiled()
        if comp.max_site >= self.Nmodes:
            raise ValueError("the operator acts on sites beyond the state's lattice")
        ns = samples.nsamples
        out = torch.empty(ns, dtype=torch.float64, device=self._dev)
        if self._model.kind == "rbm" and self._sym is None:
            self._model.eloc(self._table, comp, samples.packed, out)
            return out
        out_im = torch.empty(ns, dtype=torch.float64, device=self._dev) if self.is_complex else None
        max_conn = len(comp.host["f1"]) + len(comp.host["f2"])
        if self._model.kind == "rbm":
            ws = self.workspace("eloc", self._model.eloc_symm_workspace_bytes(ns, max_conn, self._sym))
            self._model.eloc_symm(self._table, comp, samples.packed, out, out_im, ws, self._sym)
        else:
            ws = self.workspace("eloc", self._model.eloc_workspace_bytes(ns, max_conn, self._sym))
            self._model.eloc(self._table, comp, samples.packed, out, out_im, ws, self._sym)
        return torch.complex(out, out_im) if out_im is not None else out

    def jacobian(self, s) -> torch.Tensor:
        """O_sk = d log psi(s) / d theta_k, (ns, nparams) float32 or complex64
        (variational.py:497-511)."""
        packed = s if isinstance(s, torch.Tensor) and s.dtype == torch.int32 else pack_spins(s, self.Nmodes)
        ns = packed.shape[0]
        out = self.jacobian_rows(packed, torch.empty((self.obar_rows(ns), self.nparams), dtype=torch.float32,
                                                     device=self._dev))
        return torch.complex(out[:ns], out[ns:]) if self.is_complex else out

    def jacobian_rows(self, packed: torch.Tensor, out: torch.Tensor) -> torch.Tensor:
        """O of packed configurations written into out (obar_rows(ns) x nparams float32, any row
        stride): the rows [Re O; Im O] for complex output."""
        ns = packed.shape[0]
        if self._model.kind == "rbm" and self._sym is None:
            self._model.jacobian(self._table, packed, out)
            return out
        if self._model.kind == "rbm":
            ws = self.workspace("jac", self._model.jacobian_symm_workspace_bytes(ns, self._sym))
            self._model.jacobian_symm(self._table, packed, out[:ns], out[ns:] if self.is_complex else None,
                                      out.stride(0), ws, self._sym)
            return out
        ws = self.workspace("jac", self._model.jacobian_workspace_bytes(ns, self._sym))
        self._model.jacobian(self._table, packed, out[:ns], out[ns:] if self.is_complex else None, out.stride(0), ws,
                             self._sym)
        return out

    def obar_rows(self, ns: int) -> int:
        """Rows of the matrix QNGD.solve works on: 2 ns ([Re; Im]) for complex output."""
        return 2 * ns if self.is_complex else ns

    def obar(self, samples, out: Optional[torch.Tensor] = None):
        """Centred and scaled Obar and the weighted mean Omean (sr.py:76-88); for complex
        output the rows are [Re Obar; Im Obar] as QNGD.solve stacks them (sr.py:99-105)."""
        ns = samples.nsamples
        if out is None:
            out = torch.empty((self.obar_rows(ns), self.nparams), dtype=torch.float32, device=self._dev)
        if self._model.kind == "rbm" and self._sym is None:
            omean = torch.empty(self.nparams, dtype=torch.float64, device=self._dev)
            ws = self.workspace("obar", self._model.obar_workspace_bytes(ns))
            self._model.obar(self._table, samples.packed, samples.reweight_factor, out, omean, ws)
            return out, omean
        cplx = self.is_complex
        ld = out.stride(0)
        self.jacobian_rows(samples.packed, out)
        cws = self.workspace("center", _lib.lib().qgx_center_columns_workspace_bytes(ns, self.nparams))
        halves = [out[:ns], out[ns:]] if cplx else [out]
        means = []
        for h in halves:
            m = torch.empty(self.nparams, dtype=torch.float64, device=self._dev)
            _lib.call("qgx_center_columns", _lib.ptr(h), ns, self.nparams, ld,
                      _lib.ptr(samples.reweight_factor), _lib.ptr(m), _lib.ptr(cws), cws.numel(), _lib.stream_ptr())
            means.append(m)
        omean = torch.complex(means[0], means[1]) if cplx else means[0]
        return out, omean

    # ---- parameter update ------------------------------------------------------------------
    def _check_last_update(self) -> None:
        if self._flag_event is not None and self._flag_event.query():
            if int(self._flag_host[0]) != 0:
                warnings.warn("Got invalid update step. The update is interrupted.")
            self._flag_event = None

    def update(self, step: torch.Tensor) -> None:
        """theta <- theta - step, skipped when step has a non-finite entry
        (variational.py:558-579). The skip is reported by a warning at the next update."""
        self._check_last_update()
        if step.is_complex():
            step = step.real
        step = step.to(device=self._dev, dtype=torch.float64).contiguous()
        if step.numel() != self.nparams:
            raise ValueError(f"step has {step.numel()} entries, the state has {self.nparams} parameters")
        _lib.call("qgx_apply_update", _lib.ptr(self._params), _lib.ptr(step), self.nparams, _lib.ptr(self._flag),
                  _lib.stream_ptr())
        self._flag_host.copy_(self._flag, non_blocking=True)
        self._flag_event = torch.cuda.Event()
        self._flag_event.record()
        self._refresh()

    def last_update_skipped(self) -> bool:
        """Synchronises and tells whether the last update was skipped (non-finite step)."""
        torch.cuda.current_stream().synchronize()
        self._flag_event = None
        return int(self._flag_host[0]) != 0

    def get_params_flatten(self) -> torch.Tensor:
        return self._params.clone()

    def set_params(self, params) -> None:
        p = torch.as_tensor(params, dtype=torch.float32).reshape(-1)
        if p.numel() != self.nparams:
            raise ValueError("wrong number of parameters")
        self._params.copy_(p.to(self._dev))
        self._refresh()

    def save(self, file) -> None:
        """The parameters in the reference's checkpoint format (variational.py:581-587):
        quantax loads the file with Variational(model, file), and so does this class."""
        from .checkpoint import save_model
        save_model(file, self._model, self._params.cpu().numpy())
