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

Failures stay with the job that has them (the reference's own guard is the skipped
non-finite update, quantax/state/variational.py:570-573): a spec that cannot run is refused at
submission with a "rejected: ..." status, a job whose parameters or energy turn non-finite is
retired with a "failed: ..." status (checked without stalling the other jobs: the energy of a
step is read once that step's end event has completed), and cancel(name) retires a job at its
next step boundary with the status "cancelled". Every retired job releases its memory; the
other jobs run on unchanged.
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
    init_params: Optional[np.ndarray] = None  # host parameters to start from (default: the model's init)

    def validate(self) -> None:
        """Raise ValueError when the job cannot run."""
        if self.kind not in ("tfim", "j1j2"):
            raise ValueError(f"unknown job kind {self.kind!r}")
        if self.nsamples <= 0 or self.steps <= 0:
            raise ValueError("nsamples and steps must be positive")
        if self.kind == "tfim" and not (2 <= self.L <= 128 and self.alpha >= 1):
            raise ValueError(f"tfim chain length {self.L} / alpha {self.alpha} outside 2..128 / >= 1")
        if self.kind == "j1j2":
            if not (3 <= self.L <= 16) or (self.L * self.L) % 2:
                raise ValueError(f"j1j2 needs an even number of sites on an L x L square, 3 <= L <= 16, got {self.L}")
            if not (1 <= self.blocks <= 16) or self.channels not in (2, 4, 6, 8, 10, 12, 14, 16):
                raise ValueError(f"ResConv with {self.blocks} blocks / {self.channels} channels is not supported")
        if self.conv not in ("fp32", "tf32", "bf16") or self.gram not in ("fp32", "tf32", "bf16", "3xtf32"):
            raise ValueError(f"arithmetic conv={self.conv!r} gram={self.gram!r} not supported")
        if self.solve not in ("fp64", "fp64_lib", "mixed"):
            raise ValueError(f"solve {self.solve!r} not supported")
        if self.init_params is not None:
            p = np.asarray(self.init_params)
            if p.shape != (self.nparams(),):
                raise ValueError(f"init_params has shape {p.shape}, the model has {self.nparams()} parameters")
            if not np.all(np.isfinite(p)):
                raise ValueError("init_params holds non-finite values")

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
            if spec.init_params is not None:
                self.state.set_params(torch.as_tensor(np.asarray(spec.init_params, dtype=np.float32)))
                self.sampler.reset()
            self.opt = qtx.optimizer.SR(self.state, H, solver=solver, gram=spec.gram)
            global_defs.set_default_dtype(np.float64)
        self.status = "ok"
        self._checked = 0  # steps whose energy has been checked for finiteness
        self._host_energy: List[torch.Tensor] = []
        self._e0 = None    # the running step's start event
        self._pre = None   # (samples, local energies) of the running step from a batched launch

    @property
    def batchable(self) -> bool:
        """Whether the job's sweeps and local energies can share launches with other jobs'
        (RBM states: qgx_rbm_sweep_batched / qgx_rbm_eloc_batched)."""
        return self.spec.kind == "tfim"

    def begin(self) -> None:
        """Mark the start of the next SR step on the job's stream (step() does it when not done)."""
        with torch.cuda.stream(self.stream):
            self._e0 = torch.cuda.Event(enable_timing=True)
            self._e0.record()

    @property
    def done(self) -> bool:
        return self.step_index >= self.spec.steps

    def step(self) -> None:
        """Enqueue one SR step on the job's stream (returns without waiting). A step whose sweep
        and local energies came from a batched launch (VMCServer._batched_front) starts from
        them."""
        if self._e0 is None:
            self.begin()
        with torch.cuda.stream(self.stream):
            e0, self._e0 = self._e0, None
            e1 = torch.cuda.Event(enable_timing=True)
            if self._pre is not None:
                (samples, E), self._pre = self._pre, None
                step = self.opt.get_step(samples, E)
            else:
                samples = self.sampler.sweep()
                step = self.opt.get_step(samples)
            self.state.update(step * self.spec.lr)
            self.stats.append(self.opt.stats.clone())
            host = torch.empty(1, dtype=torch.float64).pin_memory()
            host.copy_(self.stats[-1][:1], non_blocking=True)  # the energy, read once e1 has completed
            self._host_energy.append(host)
            e1.record()
            self._events.append((e0, e1))
        self.step_index += 1

    def poll_finite(self) -> bool:
        """Check the energies of the steps that have completed on the device (no waiting);
        False once one is not finite (the job's status then says which step)."""
        while self._checked < len(self._events) and self._events[self._checked][1].query():
            e = float(self._host_energy[self._checked][0])
            if not np.isfinite(e):
                self.status = f"failed: non-finite energy at step {self._checked}"
                return False
            self._checked += 1
        return True

    def finish(self) -> dict:
        self.stream.synchronize()
        self.latencies = [a.elapsed_time(b) for a, b in self._events]
        energies = [float(x[0]) for x in self.stats]
        if self.status == "ok" and not all(np.isfinite(energies)):
            self.status = f"failed: non-finite energy at step {int(np.argmin(np.isfinite(energies)))}"
        return {"name": self.spec.name, "status": self.status, "energies": energies,
                "latencies_ms": self.latencies, "samples": self.spec.nsamples * len(energies)}


@dataclass(order=True)
class _Pending:
    arrival: float
    order: int
    spec: JobSpec = field(compare=False)


class VMCServer:
    """Admits jobs by HBM budget, runs their SR steps interleaved on per-job streams."""

    def __init__(self, hbm_budget_bytes: Optional[int] = None, max_active: int = 16, batch: bool = True):
        if hbm_budget_bytes is None:
            free, _ = torch.cuda.mem_get_info()
            hbm_budget_bytes = int(free * 0.8)
        self.budget = int(hbm_budget_bytes)
        self.max_active = max_active
        self._pending: List[_Pending] = []
        self._order = 0
        self._rejected: List[dict] = []
        self._cancel = set()
        self.batch = batch  # batched sweeps and local energies of the RBM jobs of a round
        self._batch_stream = None
        self.batched_rounds = 0

    def submit(self, spec: JobSpec) -> str:
        """Queue a job; returns "queued", or "rejected: <reason>" for a spec that cannot run
        (the job then appears in run()'s results with that status). A job larger than the whole
        budget raises ValueError: no admission order could ever run it."""
        try:
            spec.validate()
        except ValueError as e:
            status = f"rejected: {e}"
            self._rejected.append({"name": spec.name, "status": status, "energies": [], "latencies_ms": [],
                                   "samples": 0})
            return status
        if spec.hbm_bytes() > self.budget:
            raise ValueError(f"job {spec.name} needs ~{spec.hbm_bytes() >> 20} MiB, above the whole budget")
        heapq.heappush(self._pending, _Pending(spec.arrival, self._order, spec))
        self._order += 1
        return "queued"

    def _batched_front(self, jobs: List[Job]) -> None:
        """The sweeps and local energies of this round's RBM jobs in shared launches, on a
        stream that waits for each job's previous step; each job's stream then waits for them,
        and the job's own step goes on from its samples and local energies."""
        from .operator import Operator
        from .sampler import Metropolis
        if self._batch_stream is None:
            self._batch_stream = torch.cuda.Stream()
        bs = self._batch_stream
        for job in jobs:
            job.begin()
            ready = torch.cuda.Event()
            ready.record(job.stream)
            bs.wait_event(ready)
        with torch.cuda.stream(bs):
            samples = Metropolis.sweep_batched([job.sampler for job in jobs])
            energies = Operator.Oloc_batched([(job.opt.hamiltonian, job.state, smp)
                                              for job, smp in zip(jobs, samples)])
            done = torch.cuda.Event()
            done.record()
        for job, smp, E in zip(jobs, samples, energies):
            job.stream.wait_event(done)
            # made on the batch stream, used on the job's: not reused before the job is done
            for t in (smp.packed, smp.log_psi, smp.reweight_factor, E):
                if isinstance(t, torch.Tensor):
                    t.record_stream(job.stream)
            job._pre = (smp, E)
        self.batched_rounds += 1

    def cancel(self, name: str) -> None:
        """Retire the job at its next step boundary (or drop it if it has not started)."""
        self._cancel.add(name)

    def run(self, on_round=None) -> dict:
        """Serve every submitted job; returns per-job results and aggregate figures.
        on_round(server, active_jobs), if given, runs after every round of step launches."""
        active: List[Job] = []
        used = 0
        results = list(self._rejected)
        self._rejected = []
        t0 = time.perf_counter()
        streams: List[torch.cuda.Stream] = []
        while self._pending or active:
            for p in [p for p in self._pending if p.spec.name in self._cancel]:
                self._pending.remove(p)
                results.append({"name": p.spec.name, "status": "cancelled", "energies": [], "latencies_ms": [],
                                "samples": 0})
            heapq.heapify(self._pending)
            if not self._pending and not active:
                break
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
            batch = [job for job in active if job.batchable] if self.batch else []
            if len(batch) >= 2:
                self._batched_front(batch)
            for job in active:
                job.step()
            if on_round is not None:
                on_round(self, active)
            still = []
            for job in active:
                if job.spec.name in self._cancel:
                    job.status = "cancelled"
                elif not job.poll_finite():
                    pass  # status says which step
                if job.done or job.status != "ok":
                    results.append(job.finish())
                    used -= job.used
                    streams.append(job.stream)
                    del job.state, job.sampler, job.opt
                else:
                    still.append(job)
            active = still
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        done = [r for r in results if r["status"] == "ok"]
        lat = sorted(x for r in done for x in r["latencies_ms"])
        pct = lambda q: lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))] if lat else None
        return {"jobs": results, "wall_s": wall, "jobs_per_s": len(done) / wall,
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
