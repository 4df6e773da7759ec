"""One MinSR step with the Markov chains split over ranks.

The reference shards its samples over devices (quantax/utils/function.py:188-245, shard_vmap)
after checking that the sample count divides evenly (quantax/sampler/sampler.py:29-33), and
lets the Gram product reduce over the devices (quantax/optimizer/solver.py:134-139). Here every
rank runs its own chains and computes the local energies E_r (n_r) and log-derivatives O_r
(n_r x Np) of its samples; one SR iteration then needs one exchange step:

  1. all-reduce of sum E, sum |E - Emean|^2 and the column sums of O: the energy, its variance
     and Omean over all Ns samples (quantax/optimizer/sr.py:76-88, 180-195);
  2. every rank centres its own rows, Obar_r = (O_r - Omean) / sqrt(Ns) and
     Ebar_r = (E_r - Emean) / sqrt(Ns);
  3. all-gather of the Obar row blocks: every rank forms its block row T_r = Obar_r Obar^T
     (n_r x Ns) of T = Obar Obar^T;
  4. all-gather of the block rows and of Ebar: every rank holds T + shift I and solves it
     (the same deterministic solve on every rank, so every rank holds the same y);
  5. x = sum_r Obar_r^T y_r by an all-reduce: the step every rank applies to its copy of the
     parameters.

Real parameters with a complex psi stack [Re; Im] rows as QNGD.solve does (sr.py:90-113); each
rank stacks its own rows, so the global rows are [Re_0; Im_0; Re_1; Im_1; ...]: a permutation
of the single-process order applied alike to T's rows and columns and to the right-hand side,
which leaves the shift (a multiple of the trace) and x = A^T y unchanged.

The block-row Gram and the projection are plain GEMMs (torch.matmul on the rank's device, a
library GEMM); the solve is injectable, by default the library's FP64 Cholesky (qgx_sym_solve)
for GPU tensors and torch's Cholesky for CPU tensors. Collectives use torch.distributed (NCCL on GPUs,
gloo on CPU); a single process is the world-size-1 case.
"""
from __future__ import annotations

import math
from typing import Callable, Optional

import torch
import torch.distributed as dist

from . import replicas


def check_divisible(nsamples: int, world: int) -> None:
    """The reference's requirement (sampler.py:29-33): every rank gets the same number of samples."""
    if nsamples % world:
        raise ValueError(f"{nsamples} samples cannot be split evenly over {world} ranks; "
                         "choose a sample count divisible by the number of ranks")


def _all_reduce(t: torch.Tensor) -> torch.Tensor:
    if replicas.world() > 1:
        dist.all_reduce(t)
    return t


def _all_gather_rows(t: torch.Tensor) -> torch.Tensor:
    w = replicas.world()
    if w == 1:
        return t
    parts = [torch.empty_like(t) for _ in range(w)]
    dist.all_gather(parts, t.contiguous())
    return torch.cat(parts, dim=0)


def cholesky_solve(T: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """y = T^-1 b by an FP64 Cholesky (the shifted T is symmetric positive definite)."""
    L = torch.linalg.cholesky(T)
    return torch.cholesky_solve(b.unsqueeze(1), L).squeeze(1)


def device_cholesky_solve(T: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """The library's FP64 Cholesky solve of a given matrix (qgx_sym_solve, QGX_SOLVE_SHIFT with
    no further shift) on the GPU the tensors live on; T is not modified."""
    import ctypes as C
    from . import _lib
    n = T.shape[0]
    S = T.to(torch.float64).contiguous().clone()
    f = b.to(torch.float64).contiguous()
    nbytes = C.c_int64(0)
    _lib.call("qgx_solve_workspace_bytes", n, 1, _lib.SOLVE_SHIFT, C.byref(nbytes))
    ws = torch.empty(max(nbytes.value, 256), dtype=torch.uint8, device=T.device)
    x = torch.empty(n, dtype=torch.float64, device=T.device)
    _lib.call("qgx_sym_solve", _lib.ptr(S), n, _lib.ptr(f), _lib.SOLVE_SHIFT, 0.0, 0.0, 0.0, 0.0, _lib.ptr(x), None,
              _lib.ptr(ws), ws.numel(), _lib.stream_ptr())
    return x


class ShardedMinSR:
    """The MinSR step of minnorm_shift_eig(rshift, ashift) (solver.py:50-62) over chain-sharded
    samples. `solve(T, b)` solves the already shifted system; by default the library's FP64
    Cholesky on a GPU and torch's on the CPU."""

    def __init__(self, rshift: float = 1e-12, ashift: float = 1e-4,
                 solve: Optional[Callable[[torch.Tensor, torch.Tensor], torch.Tensor]] = None):
        self.rshift, self.ashift = float(rshift), float(ashift)
        self._solve = solve
        self.energy = float("nan")
        self.VarE = float("nan")

    def step(self, O_local: torch.Tensor, E_local: torch.Tensor) -> torch.Tensor:
        """O_local (n_r x Np, real or complex), E_local (n_r): this rank's samples. Returns the
        step x (Np, float64), identical on every rank."""
        world = replicas.world()
        n_r = O_local.shape[0]
        ns = n_r * world
        check_divisible(ns, world)
        O = O_local.to(torch.complex128 if O_local.is_complex() else torch.float64)
        E = E_local.to(torch.complex128)
        # 1. global statistics
        sums = torch.cat([torch.view_as_real(E.sum().reshape(1)).reshape(2), torch.view_as_real(
            O.sum(dim=0).to(torch.complex128)).reshape(-1)])
        _all_reduce(sums)
        emean = torch.complex(sums[0], sums[1]) / ns
        omean = torch.view_as_complex(sums[2:].reshape(-1, 2)) / ns
        dev2 = (E - emean).abs().pow(2).sum().reshape(1)
        _all_reduce(dev2)
        self.energy = float(emean.real)
        self.VarE = float(dev2 / ns)
        # 2. centre this rank's rows; [Re; Im] stacking for complex O
        scale = 1.0 / math.sqrt(ns)
        ob = (O - (omean if O.is_complex() else omean.real)) * scale
        eb = (E - emean) * scale
        if O.is_complex():
            A_r = torch.cat([ob.real, ob.imag], dim=0)
            b_r = torch.cat([eb.real, eb.imag])
        else:
            A_r, b_r = ob, eb.real
        # 3. every rank's block row of T = A A^T
        A_all = _all_gather_rows(A_r)
        T_r = A_r @ A_all.T
        # 4. the whole shifted T and right-hand side on every rank, one deterministic solve
        T = _all_gather_rows(T_r)
        b = _all_gather_rows(b_r)
        tr = torch.diagonal(T).sum()
        T = T + (self.rshift * tr + self.ashift) * torch.eye(T.shape[0], dtype=T.dtype, device=T.device)
        solve = self._solve or (device_cholesky_solve if T.is_cuda else cholesky_solve)
        y = solve(T, b)
        # 5. x = sum_r A_r^T y_r
        y_r = y.reshape(world, A_r.shape[0])[replicas.rank()]
        x = A_r.T @ y_r
        return _all_reduce(x.contiguous())
