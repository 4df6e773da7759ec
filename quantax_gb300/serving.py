"""Continuous batching of independent VMC jobs on one GPU.

A job is one VMC optimisation (lattice, Hamiltonian, model, sample count, number of SR
steps, seed). The server keeps every admitted job resident on the device -- parameters,
chains, the sampler's RNG counter and all step buffers -- and gives it its own CUDA
stream, so the sweeps, local energies, Gram builds and solves of different jobs overlap on
the device. Jobs arrive over time; a job is admitted when it has arrived and its HBM
estimate fits the remaining budget, and it releases its memory when it retires, which
admits the next ones. Each SR step is bracketed by CUDA events on the job's stream; the
server reports per-step latency percentiles, jobs/s and aggregate samples/s.

A job's result does not depend on the mix: its random numbers come from its own seed
stream (Philox counters keyed per job) and every reduction has a fixed order.
"""
from __future__ import annotations

import heapq
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import torch

from . import global_defs


@dataclass
class JobSpec:
    name: str
    kind: str                 # "tfim" (chain, RBM_Dense) or "j1j2" (square, ResConv)
    L: int
    nsamples: int
    steps: int
    seed: int
    h: float = 1.0            # tfim transverse field
    alpha: int = 2            # tfim RBM hidden-unit density
    J2: float = 0.5           # j1j2 next-nearest coupling
    blocks: int = 4           # j1j2 ResConv depth
    channels: int = 8         # j1j2 ResConv width
    lr: float = 1e-2
    ashift: float = 1e-4
    conv: str = "bf16"        # ResConv forward convolutions: "fp32", "tf32" or "bf16"
    gram: str = "bf16"        # Gram matrix arithmetic: "fp32", "tf32", "bf16" or "3xtf32"
    solve: str = "fp64"
    arrival: float = 0.0      # seconds after the server starts

    def nparams(self) -> int:
        if self.kind == "tfim":
            M = self.alpha * self.L
            return M * self.L + M
        C, B = self.channels, self.blocks
        return (C * 9 + C) + (C * C * 9 + C) + (B - 1) * 2 * (C * C * 9 + C) - C

    def rows(self) -> int:
        return self.nsamples if self.kind == "tfim" else 2 * self.nsamples

    def hbm_bytes(self) -> int:
        """Estimate of the job's resident device memory (Obar, Gram, solver and sampler buffers)."""
        rows, npar = self.rows(), self.nparams()
        n = self.L if self.kind == "tfim" else self.L * self.L
        b = rows * npar * 4                        # Obar
        b += rows * rows * 8                       # Gram (FP64)
        b += rows * rows * 4 if self.solve == "mixed" else 0
        b += (rows // 256 + 1) * max(rows, npar) * 8  # projection partial sums
        if self.kind == "j1j2":
            b += self.nsamples * 400 * (4 * ((n + 31) // 32) + 16)  # connected configurations
            b += 4 * 160 * self.blocks * 2 * self.channels * n * 4  # backward scratch
        else:
            b += self.nsamples * 128 * self.alpha * self.L // 32 * 4 + 2 * (self.nsamples // 128 + 1) * npar * 8
        return int(b * 1.1) + (64 << 20)


class Job:
    def __init__(self, spec: JobSpec, stream: torch.cuda.Stream):
        import quantax_gb300 as qtx
        self.spec = spec
        self.stream = stream
        self.step_index = 0
        self.latencies: List[float] = []
        self.stats: List[torch.Tensor] = []
        self._events = []
        with torch.cuda.stream(stream):
            qtx.set_random_seed(spec.seed)
            solver = qtx.optimizer.minnorm_shift_eig(ashift=spec.ashift, precision=spec.solve)
            if spec.kind == "tfim":
                qtx.set_default_dtype(np.float64)
                qtx.sites.Chain(spec.L)
                H = qtx.operator.Ising(h=spec.h)
                self.state = qtx.state.Variational(qtx.model.RBM_Dense(spec.alpha * spec.L, init_std=0.01))
                self.sampler = qtx.sampler.LocalFlip(self.state, spec.nsamples, thermal_steps=4 * spec.L,
                                                     sweep_steps=spec.L)
            elif spec.kind == "j1j2":
                qtx.set_default_dtype(np.complex128)
                n = spec.L * spec.L
                qtx.sites.Square(spec.L, Nparticles=(n // 2, n // 2))
                H = qtx.operator.Heisenberg(J=[1.0, spec.J2], n_neighbor=[1, 2], msr=True)
                self.state = qtx.state.Variational(
                    qtx.model.ResConv(spec.blocks, spec.channels, out_dtype=np.complex64, conv_precision=spec.conv))
                self.sampler = qtx.sampler.SpinExchange(self.state, spec.nsamples, thermal_steps=n, sweep_steps=n)
            else:
                raise ValueError(spec.kind)
            self.opt = qtx.optimizer.SR(self.state, H, solver=solver, gram=spec.gram)
            global_defs.set_default_dtype(np.float64)

    @property
    def done(self) -> bool:
        return self.step_index >= self.spec.steps

    def step(self) -> None:
        """Enqueue one SR step on the job's stream (returns without waiting)."""
        with torch.cuda.stream(self.stream):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            samples = self.sampler.sweep()
            step = self.opt.get_step(samples)
            self.state.update(step * self.spec.lr)
            self.stats.append(self.opt.stats.clone())
            e1.record()
            self._events.append((e0, e1))
        self.step_index += 1

    def finish(self) -> dict:
        self.stream.synchronize()
        self.latencies = [a.elapsed_time(b) for a, b in self._events]
        energies = [float(x[0]) for x in self.stats]
        return {"name": self.spec.name, "energies": energies, "latencies_ms": self.latencies,
                "samples": self.spec.nsamples * self.spec.steps}


@dataclass(order=True)
class _Pending:
    arrival: float
    order: int
    spec: JobSpec = field(compare=False)


class VMCServer:
    """Admits jobs by HBM budget, runs their SR steps interleaved on per-job streams."""

    def __init__(self, hbm_budget_bytes: Optional[int] = None, max_active: int = 16):
        if hbm_budget_bytes is None:
            free, _ = torch.cuda.mem_get_info()
            hbm_budget_bytes = int(free * 0.8)
        self.budget = int(hbm_budget_bytes)
        self.max_active = max_active
        self._pending: List[_Pending] = []
        self._order = 0

    def submit(self, spec: JobSpec) -> None:
        if spec.hbm_bytes() > self.budget:
            raise ValueError(f"job {spec.name} needs ~{spec.hbm_bytes() >> 20} MiB, above the whole budget")
        heapq.heappush(self._pending, _Pending(spec.arrival, self._order, spec))
        self._order += 1

    def run(self) -> dict:
        """Serve every submitted job; returns per-job results and aggregate figures."""
        active: List[Job] = []
        used = 0
        results = []
        t0 = time.perf_counter()
        streams: List[torch.cuda.Stream] = []
        while self._pending or active:
            now = time.perf_counter() - t0
            # admit arrived jobs while memory and slots allow (in arrival order)
            while (self._pending and self._pending[0].arrival <= now and len(active) < self.max_active
                   and used + self._pending[0].spec.hbm_bytes() <= self.budget):
                spec = heapq.heappop(self._pending).spec
                stream = streams.pop() if streams else torch.cuda.Stream()
                job = Job(spec, stream)
                job.used = spec.hbm_bytes()
                used += job.used
                active.append(job)
            if not active:
                time.sleep(min(0.01, max(0.0, self._pending[0].arrival - now)))
                continue
            for job in active:
                job.step()
            still = []
            for job in active:
                if job.done:
                    results.append(job.finish())
                    used -= job.used
                    streams.append(job.stream)
                    del job.state, job.sampler, job.opt
                else:
                    still.append(job)
            active = still
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        lat = sorted(x for r in results for x in r["latencies_ms"])
        pct = lambda q: lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))] if lat else None
        return {"jobs": results, "wall_s": wall, "jobs_per_s": len(results) / wall,
                "samples_per_s": sum(r["samples"] for r in results) / wall,
                "p50_step_ms": pct(0.5), "p99_step_ms": pct(0.99), "steps": len(lat)}


def poisson_jobs(n_jobs: int, seed: int, rate_per_s: float = 4.0, steps: int = 50,
                 nsamples_choices=(1024, 2048, 4096, 8192)) -> List[JobSpec]:
    """The mixed job stream of the serving workload: TFIM chains (L in {16,32,64,128},
    h ~ U[0.5, 1.5], RBM alpha in {1,2,4}) and J1-J2 squares (L in {4,6,8,10},
    J2 ~ U[0, 0.6], ResConv 4-8 blocks and 8-16 channels), sample counts drawn from
    nsamples_choices, Poisson arrivals."""
    rng = np.random.default_rng(seed)
    t = 0.0
    jobs = []
    for k in range(n_jobs):
        t += rng.exponential(1.0 / rate_per_s)
        ns = int(rng.choice(nsamples_choices))
        if rng.random() < 0.5:
            jobs.append(JobSpec(f"tfim{k}", "tfim", int(rng.choice([16, 32, 64, 128])), ns, steps,
                                int(rng.integers(1 << 31)), h=float(rng.uniform(0.5, 1.5)),
                                alpha=int(rng.choice([1, 2, 4])), arrival=t))
        else:
            jobs.append(JobSpec(f"j1j2_{k}", "j1j2", int(rng.choice([4, 6, 8, 10])), ns, steps,
                                int(rng.integers(1 << 31)), J2=float(rng.uniform(0.0, 0.6)),
                                blocks=int(rng.integers(4, 9)), channels=int(rng.choice([8, 12, 16])), arrival=t))
    return jobs
