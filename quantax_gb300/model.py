"""Variational models and their device kernels.

RBM_Dense mirrors quantax/model/shallow_nets.py:35-126: psi(s) = prod_i cosh(W s + b)_i,
optionally times exp(a.s) (a visible bias, absent in the reference). Parameters are
flattened in the reference's ravel order: W (M x N, row-major), b (M), then a (N).

ResConv mirrors quantax/model/conv_nets.py:95-183 (residual CNN, 3x3 circular
convolutions, tanh-GELU, mean-exp pooling, optional complex output via pair_cpl).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np
import torch

from . import _lib
from .global_defs import get_sites, get_subkeys


def _truncated_normal(rng, shape, std):
    """Normal(0, std^2) truncated at +-2 std, rescaled to unit variance like JAX's
    variance_scaling("truncated_normal") (quantax/nn/initializers.py:29-57)."""
    out = rng.standard_normal(shape)
    bad = np.abs(out) > 2.0
    while bad.any():
        out[bad] = rng.standard_normal(int(bad.sum()))
        bad = np.abs(out) > 2.0
    return out * std / 0.87962566103423978


def _cosh_scale(features: int, n_sites: int, rng) -> float:
    """Grid search of quantax/model/shallow_nets.py:17-32 for cosh: the scale in [0, 1)
    whose output std over 1000 normal inputs is closest to 0.1 sqrt(N)."""
    x = rng.standard_normal((1000, features))
    target = 0.1 * np.sqrt(n_sites)
    best, arg = np.inf, 0.0
    for scale in np.arange(0, 1, 0.01):
        out = np.sum(np.log(np.abs(np.cosh(x * scale))), axis=1)
        err = (np.std(out) - target) ** 2
        if err < best:
            best, arg = err, scale
    return float(arg)


class RBM_Dense:
    """Restricted Boltzmann machine with one dense layer, psi = prod cosh(W s + b)."""

    kind = "rbm"
    holomorphic = False

    def __init__(self, features: int, use_bias: bool = True, dtype=np.float32, visible_bias: bool = False,
                 init_std: Optional[float] = None, seed: Optional[int] = None):
        if np.dtype(dtype) != np.float32:
            raise NotImplementedError("RBM_Dense runs with float32 parameters")
        sites = get_sites()
        self.N = sites.Nmodes
        self.M = int(features)
        self.use_bias = use_bias
        self.visible_bias = visible_bias
        rng = np.random.default_rng(get_subkeys() if seed is None else seed)
        if init_std is not None:
            W = rng.normal(0.0, init_std, (self.M, self.N))
            b = rng.normal(0.0, init_std, self.M) if use_bias else np.zeros(self.M)
            a = rng.normal(0.0, init_std, self.N) if visible_bias else None
        else:
            W = _truncated_normal(rng, (self.M, self.N), 1.0 / np.sqrt(self.N))
            W *= _cosh_scale(self.M, self.N, rng)
            b = np.zeros(self.M)
            a = np.zeros(self.N) if visible_bias else None
        parts = [W.ravel(), b] + ([a] if a is not None else [])
        self.init_params = np.concatenate(parts).astype(np.float32)

    @property
    def nparams(self) -> int:
        return self.M * self.N + self.M + (self.N if self.visible_bias else 0)

    def param_blocks(self) -> list:
        """Parameter counts of the layers that hold parameters (one Linear layer)."""
        return [self.nparams]

    @classmethod
    def from_arrays(cls, W, b, a=None):
        """Model with explicit parameters (W (M, N), b (M), optional a (N))."""
        obj = cls.__new__(cls)
        W = np.asarray(W, np.float32)
        obj.M, obj.N = W.shape
        obj.use_bias = True
        obj.visible_bias = a is not None
        parts = [W.ravel(), np.asarray(b, np.float32)] + ([np.asarray(a, np.float32)] if a is not None else [])
        obj.init_params = np.concatenate(parts).astype(np.float32)
        return obj

    # ---- device side ------------------------------------------------------------------------
    def table_floats(self) -> int:
        return int(_lib.lib().qgx_rbm_table_floats(self.N, self.M))

    def split(self, params: torch.Tensor):
        M, N = self.M, self.N
        W = params[:M * N]
        b = params[M * N:M * N + M]
        a = params[M * N + M:] if self.visible_bias else None
        return W, b, a

    def prepare(self, params: torch.Tensor, table: torch.Tensor) -> None:
        W, b, a = self.split(params)
        _lib.call("qgx_rbm_prepare", _lib.ptr(W), _lib.ptr(b), _lib.ptr(a), self.N, self.M, _lib.ptr(table),
                  _lib.stream_ptr())

    def log_psi(self, table, packed, out):
        _lib.call("qgx_rbm_log_psi", _lib.ptr(table), self.N, self.M, _lib.ptr(packed), packed.shape[0],
                  _lib.ptr(out), _lib.stream_ptr())

    def sweep(self, table, packed, log_psi, accepts, nsteps, seed, step0, reweight, proposal, nbr, z, hop):
        _lib.call("qgx_rbm_sweep", _lib.ptr(table), self.N, self.M, _lib.ptr(packed), _lib.ptr(log_psi),
                  _lib.ptr(accepts), packed.shape[0], int(nsteps), int(seed), int(step0), float(reweight),
                  int(proposal), _lib.ptr(nbr), int(z), int(hop), _lib.stream_ptr())

    def eloc(self, table, compiled_op, packed, out):
        _lib.call("qgx_rbm_eloc", _lib.ptr(table), self.N, self.M, C.byref(compiled_op.struct), _lib.ptr(packed),
                  packed.shape[0], _lib.ptr(out), _lib.stream_ptr())

    def jacobian(self, table, packed, out):
        _lib.call("qgx_rbm_jacobian", _lib.ptr(table), self.N, self.M, int(self.visible_bias), _lib.ptr(packed),
                  packed.shape[0], _lib.ptr(out), out.stride(0), _lib.stream_ptr())

    def obar_workspace_bytes(self, ns: int) -> int:
        return int(_lib.lib().qgx_rbm_obar_workspace_bytes(self.N, self.M, ns))

    # ---- the projected state (symm: a non-identity quantax_gb300.symmetry.Symmetry) ---------
    def log_psi_symm_workspace_bytes(self, ns, symm):
        return int(_lib.lib().qgx_rbm_log_psi_symm_workspace_bytes(self.N, ns, symm.nsymm))

    def log_psi_symm(self, table, packed, out, symm, workspace):
        """log psi_symm as (re, im) pairs into out ((ns, 2) float32)."""
        _lib.call("qgx_rbm_log_psi_symm", _lib.ptr(table), self.N, self.M, C.byref(symm.device_struct()),
                  _lib.ptr(packed), packed.shape[0], _lib.ptr(out), _lib.ptr(workspace), workspace.numel(),
                  _lib.stream_ptr())

    def sweep_symm_workspace_bytes(self, ns, symm):
        return int(_lib.lib().qgx_rbm_sweep_symm_workspace_bytes(self.N, ns, symm.nsymm))

    def sweep_symm(self, table, packed, log_psi, accepts, nsteps, seed, step0, reweight, proposal, nbr, z, hop,
                   workspace, symm):
        _lib.call("qgx_rbm_sweep_symm", _lib.ptr(table), self.N, self.M, C.byref(symm.device_struct()),
                  _lib.ptr(packed), _lib.ptr(log_psi), _lib.ptr(accepts), packed.shape[0], int(nsteps), int(seed),
                  int(step0), float(reweight), int(proposal), _lib.ptr(nbr), int(z), int(hop), _lib.ptr(workspace),
                  workspace.numel(), _lib.stream_ptr())

    def eloc_symm_workspace_bytes(self, ns, max_conn, symm):
        return int(_lib.lib().qgx_rbm_eloc_symm_workspace_bytes(self.N, ns, max_conn, symm.nsymm))

    def eloc_symm(self, table, compiled_op, packed, out_re, out_im, workspace, symm):
        _lib.call("qgx_rbm_eloc_symm", _lib.ptr(table), self.N, self.M, C.byref(symm.device_struct()),
                  C.byref(compiled_op.struct), _lib.ptr(packed), packed.shape[0], _lib.ptr(out_re), _lib.ptr(out_im),
                  _lib.ptr(workspace), workspace.numel(), _lib.stream_ptr())

    def jacobian_symm_workspace_bytes(self, ns, symm):
        return int(_lib.lib().qgx_rbm_jacobian_symm_workspace_bytes(self.N, self.M, int(self.visible_bias), ns,
                                                                      symm.nsymm))

    def jacobian_symm(self, table, packed, o_re, o_im, ldo, workspace, symm):
        _lib.call("qgx_rbm_jacobian_symm", _lib.ptr(table), self.N, self.M, int(self.visible_bias),
                  C.byref(symm.device_struct()), _lib.ptr(packed), packed.shape[0], _lib.ptr(o_re), _lib.ptr(o_im),
                  int(ldo), _lib.ptr(workspace), workspace.numel(), _lib.stream_ptr())

    def obar(self, table, packed, r, out, omean, workspace):
        _lib.call("qgx_rbm_obar", _lib.ptr(table), self.N, self.M, int(self.visible_bias), _lib.ptr(packed),
                  _lib.ptr(r), packed.shape[0], _lib.ptr(out), out.stride(0), _lib.ptr(omean), _lib.ptr(workspace),
                  workspace.numel(), _lib.stream_ptr())


class RBM_Conv(RBM_Dense):
    """Restricted Boltzmann machine with one convolutional layer (quantax/model/shallow_nets.py:
    129-190): psi = prod cosh(Conv(s)), a circular convolution whose kernel covers the whole
    (periodic) lattice. Parameters in the reference's ravel order: the kernel (channels x
    lattice shape, row-major), then the biases. The device evaluates it as the dense RBM with
    channels x Nsites hidden units that the kernel's translated copies make."""

    conv = True

    def __init__(self, channels: int, use_bias: bool = True, dtype=np.float32, init_std: Optional[float] = None,
                 seed: Optional[int] = None):
        from .global_defs import get_lattice
        if np.dtype(dtype) != np.float32:
            raise NotImplementedError("RBM_Conv runs with float32 parameters")
        lat = get_lattice()
        if lat.ndim > 2 or lat.shape[0] != 1:
            raise NotImplementedError("RBM_Conv: 1D and 2D lattices with one site per cell")
        dims = tuple(lat.shape[1:]) + ((1,) if lat.ndim == 1 else ())
        self.L0, self.L1 = int(dims[0]), int(dims[1])
        self.channels = int(channels)
        self.N = self.L0 * self.L1
        self.M = self.channels * self.N  # hidden units of the equivalent dense RBM
        if self.M > 2048:
            raise NotImplementedError("RBM_Conv: channels x Nsites <= 2048")
        self.use_bias = use_bias
        self.visible_bias = False
        rng = np.random.default_rng(get_subkeys() if seed is None else seed)
        shape = (self.channels, self.N)
        if init_std is not None:
            W = rng.normal(0.0, init_std, shape)
            b = rng.normal(0.0, init_std, self.channels) if use_bias else np.zeros(self.channels)
        else:
            # lecun normal (fan-in = the kernel's size), then the cosh output scale of
            # shallow_nets.py:17-32 over channels x cells features (:174-176); zero biases
            W = _truncated_normal(rng, shape, 1.0 / np.sqrt(self.N)) * _cosh_scale(self.M, self.N, rng)
            b = np.zeros(self.channels)
        self.init_params = np.concatenate([W.ravel(), b]).astype(np.float32)

    @property
    def nparams(self) -> int:
        return self.channels * self.N + self.channels

    def table_floats(self) -> int:
        return int(_lib.lib().qgx_rbm_conv_table_floats(self.L0, self.L1, self.channels))

    def prepare(self, params: torch.Tensor, table: torch.Tensor) -> None:
        _lib.call("qgx_rbm_conv_prepare", _lib.ptr(params), self.L0, self.L1, self.channels, _lib.ptr(table),
                  _lib.stream_ptr())

    def jacobian(self, table, packed, out):
        _lib.call("qgx_rbm_conv_jacobian", _lib.ptr(table), self.L0, self.L1, self.channels, _lib.ptr(packed),
                  packed.shape[0], _lib.ptr(out), out.stride(0), _lib.stream_ptr())

    def obar_workspace_bytes(self, ns: int) -> int:
        return int(_lib.lib().qgx_center_columns_workspace_bytes(ns, self.nparams))

    def obar(self, table, packed, r, out, omean, workspace):
        """Obar = (O - <O>) sqrt(r / Ns): the log-derivatives, then the column centring."""
        self.jacobian(table, packed, out)
        _lib.call("qgx_center_columns", _lib.ptr(out), packed.shape[0], self.nparams, out.stride(0), _lib.ptr(r),
                  _lib.ptr(omean), _lib.ptr(workspace), workspace.numel(), _lib.stream_ptr())


class ResConv:
    """Deep convolutional residual network (conv_nets.py:95-183) on a periodic L x L lattice."""

    kind = "resconv"
    holomorphic = False

    def __init__(self, nblocks: int, channels: int, kernel_size: int = 3, final_activation=None, trans_symm=None,
                 dtype=np.float32, out_dtype=None, seed: Optional[int] = None, conv_precision: str = "fp32"):
        """conv_precision: arithmetic of the forward convolutions used by sampling and local
        energies -- "fp32" (CUDA cores), "tf32" or "bf16" (tensor-core operands, FP32
        accumulation). The log-derivatives are always computed in FP32."""
        from . import nn
        from .global_defs import get_lattice
        if kernel_size != 3 or trans_symm is not None:
            raise NotImplementedError("quantax_gb300 ResConv: 3x3 kernels and the default translation "
                                      "symmetrisation only")
        if final_activation not in (None, nn.exp_by_scale, nn.sinhp1_by_scale):
            raise NotImplementedError("ResConv final_activation: quantax_gb300.nn.exp_by_scale or sinhp1_by_scale")
        self.sinhp1 = final_activation is nn.sinhp1_by_scale
        if np.dtype(dtype) != np.float32:
            raise NotImplementedError("ResConv runs with float32 parameters")
        lat = get_lattice()
        if lat.ndim != 2 or lat.shape[1] != lat.shape[2] or not np.all(lat.boundary == 1):
            raise NotImplementedError("ResConv needs a periodic square lattice")
        self.L = lat.shape[1]
        self.N = lat.Nsites
        self.nblocks = int(nblocks)
        self.channels = int(channels)
        self.complex_output = out_dtype is not None and np.issubdtype(np.dtype(out_dtype), np.complexfloating)
        self.conv_precision = conv_precision
        rng = np.random.default_rng(get_subkeys() if seed is None else seed)
        parts = []
        for b in range(self.nblocks):
            for layer in range(2):
                cin = 1 if (b == 0 and layer == 0) else self.channels
                w = _truncated_normal(rng, (self.channels, cin, 3, 3), np.sqrt(2.0 / (cin * 9)))  # He normal
                parts.append(w.ravel())
                if not (layer == 1 and b == self.nblocks - 1):
                    parts.append(np.zeros(self.channels))
        self.init_params = np.concatenate(parts).astype(np.float32)

    @property
    def nparams(self) -> int:
        return int(self.init_params.size)

    def param_blocks(self) -> list:
        """Parameter counts of the layers that hold parameters: one per residual block
        (conv_nets.py:26-92; the reshape, final and symmetrising layers hold none)."""
        C, out = self.channels, []
        for b in range(self.nblocks):
            cin = 1 if b == 0 else C
            out.append(C * cin * 9 + C + C * C * 9 + (C if b != self.nblocks - 1 else 0))
        return out

    def table_floats(self) -> int:
        return int(_lib.lib().qgx_resconv_table_floats(self.nblocks, self.channels))

    def prepare(self, params, table):
        _lib.call("qgx_resconv_prepare", _lib.ptr(params), self.nblocks, self.channels, _lib.ptr(table),
                  _lib.stream_ptr())

    @property
    def conv_precision(self) -> str:
        return self._conv_precision

    @conv_precision.setter
    def conv_precision(self, p: str):
        codes = {"fp32": _lib.CONV_FP32, "tf32": _lib.CONV_TF32, "bf16": _lib.CONV_BF16}
        if p not in codes:
            raise ValueError(f"conv_precision must be one of {sorted(codes)}, got {p!r}")
        self._conv_precision = p
        self._conv_code = codes[p]

    @property
    def signed_output(self) -> bool:
        """A real output that can be negative (sinhp1): log psi carries the sign as its phase."""
        return self.sinhp1 and not self.complex_output

    def _args(self):
        flags = (_lib.RESCONV_COMPLEX if self.complex_output else 0) | (_lib.RESCONV_SINHP1 if self.sinhp1 else 0)
        return (self.L, self.nblocks, self.channels, flags)

    def _fwd_args(self):
        return self._args() + (self._conv_code,)

    # symm: a non-identity quantax_gb300.symmetry.Symmetry, or None
    def log_psi_workspace_bytes(self, ns, symm=None):
        return 0 if symm is None else int(_lib.lib().qgx_resconv_log_psi_symm_workspace_bytes(self.L, ns, symm.nsymm))

    def log_psi(self, table, packed, out, symm=None, workspace=None):
        """out: (ns, 2) float32 (re, im)."""
        if symm is None:
            _lib.call("qgx_resconv_log_psi", _lib.ptr(table), *self._fwd_args(), _lib.ptr(packed), packed.shape[0],
                      _lib.ptr(out), _lib.stream_ptr())
            return
        _lib.call("qgx_resconv_log_psi_symm", _lib.ptr(table), *self._fwd_args(), C.byref(symm.device_struct()),
                  _lib.ptr(packed), packed.shape[0], _lib.ptr(out), _lib.ptr(workspace), workspace.numel(),
                  _lib.stream_ptr())

    def sweep_workspace_bytes(self, ns, symm=None):
        if symm is None:
            return int(_lib.lib().qgx_resconv_sweep_workspace_bytes(self.L, ns))
        return int(_lib.lib().qgx_resconv_sweep_symm_workspace_bytes(self.L, ns, symm.nsymm))

    def sweep(self, table, packed, log_psi, accepts, nsteps, seed, step0, reweight, proposal, nbr, z, hop,
              workspace, symm=None):
        if proposal != _lib.PROPOSAL_SPIN_EXCHANGE:
            raise NotImplementedError("the ResConv sampler implements SpinExchange proposals")
        head = (_lib.ptr(table), *self._fwd_args())
        if symm is not None:
            head = head + (C.byref(symm.device_struct()),)
        _lib.call("qgx_resconv_sweep" if symm is None else "qgx_resconv_sweep_symm", *head, _lib.ptr(packed),
                  _lib.ptr(log_psi), _lib.ptr(accepts), packed.shape[0], int(nsteps), int(seed), int(step0),
                  float(reweight), _lib.ptr(nbr), int(z), int(hop), _lib.ptr(workspace), workspace.numel(),
                  _lib.stream_ptr())

    def eloc_workspace_bytes(self, ns, max_conn, symm=None):
        if symm is None:
            return int(_lib.lib().qgx_resconv_eloc_workspace_bytes(self.L, ns, max_conn))
        return int(_lib.lib().qgx_resconv_eloc_symm_workspace_bytes(self.L, ns, max_conn, symm.nsymm))

    def eloc(self, table, compiled_op, packed, out_re, out_im, workspace, symm=None):
        head = (_lib.ptr(table), *self._fwd_args())
        if symm is not None:
            head = head + (C.byref(symm.device_struct()),)
        _lib.call("qgx_resconv_eloc" if symm is None else "qgx_resconv_eloc_symm", *head, C.byref(compiled_op.struct),
                  _lib.ptr(packed), packed.shape[0], _lib.ptr(out_re), _lib.ptr(out_im), _lib.ptr(workspace),
                  workspace.numel(), _lib.stream_ptr())

    def jacobian_workspace_bytes(self, ns=1, symm=None):
        if symm is None:
            return int(_lib.lib().qgx_resconv_jacobian_workspace_bytes(self.L, self.nblocks, self.channels))
        return int(_lib.lib().qgx_resconv_jacobian_symm_workspace_bytes(self.L, self.nblocks, self.channels, ns,
                                                                          symm.nsymm))

    def jacobian(self, table, packed, o_re, o_im, ldo, workspace, symm=None):
        head = (_lib.ptr(table), *self._args())
        if symm is not None:
            head = head + (C.byref(symm.device_struct()),)
        _lib.call("qgx_resconv_jacobian" if symm is None else "qgx_resconv_jacobian_symm", *head, _lib.ptr(packed),
                  packed.shape[0], _lib.ptr(o_re), _lib.ptr(o_im), int(ldo), _lib.ptr(workspace), workspace.numel(),
                  _lib.stream_ptr())
