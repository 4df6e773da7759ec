#!/usr/bin/env python
"""Benchmark of the VMC inner loop on one GB300 (one JSON line on stdout).

Default workload (--workload resconv): J1-J2 Heisenberg (J2 = 0.5, MSR) on the periodic 10 x 10
square lattice in the Sz = 0 sector; ResConv with 8 residual blocks and 16 channels, complex
output (34,944 float32 parameters, He-normal init); SpinExchange with 16384 chains, 200
proposals per sweep and 200 thermalisation proposals; MinSR with diagonal shift 1e-4
(minnorm_shift_eig) on the stacked [Re; Im] 32768 x 34944 matrix. `value` is the plain method
(FP32 convolutions, FP32-class Gram, FP64 solve); `forms` holds the accurate form (the plain
arithmetic with the FP32-preconditioned FP64 solve) and the precision forms (TF32 / BF16
tensor-core convolutions and Gram) on the same seeds, each with its speed-up over the plain
method, its p50 / p99 step latency and its energies' difference from the plain run.

--workload rbm: chain L=64 periodic TFIM h=J=1; RBM_Dense with 256 hidden units (16,640 float32
parameters, N(0, 0.01^2) init); LocalFlip with 8192 chains, 64 proposals per sweep, 640
thermalisation proposals; MinSR (T 8192 x 8192) with diagonal shift 1e-4.

One step = one SR iteration: sweep, local energies, Obar, Gram, solve, parameter update.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload ...]

Under torchrun with N > 1 every rank runs an independent replica of the workload (the chains
of different replicas never interact, no collective on the data path): weak scaling; timing is
bracketed by barriers and the max over ranks is reported. --impl reference times whole SR
steps of the CPU restatement (oracle/cpu_vmc.py) on the host cores at the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "SR steps/s"
UNIT = "SR_steps/s"

# the workload as both arms report it in `config` (arithmetic choices go to `method`)
WORKLOADS = {
    "resconv": dict(workload="j1j2_square10_resconv8x16_minsr16384", lattice="Square(10) PBC, Sz=0",
                    hamiltonian="Heisenberg(J=[1, 0.5], n_neighbor=[1, 2], msr=True)",
                    wavefunction="ResConv(8 blocks, 16 channels, complex output)", nparams=34944,
                    sampler="SpinExchange", chains=16384, proposals_per_sweep=200, thermal_proposals=200,
                    solver="minnorm_shift_eig(ashift=1e-4) on the stacked [Re; Im] 32768 x 34944 matrix",
                    l2="inputs larger than L2: Obar (4.6 GB) and T (8.6 GB) exceed the 129 MB L2 every step"),
    "rbm": dict(workload="tfim_chain64_rbm256_minsr8192", lattice="Chain(64) PBC", hamiltonian="Ising(h=1, J=1)",
                wavefunction="RBM_Dense(features=256)", nparams=16640, sampler="LocalFlip", chains=8192,
                proposals_per_sweep=64, thermal_proposals=640, solver="minnorm_shift_eig(ashift=1e-4)",
                l2="inputs larger than L2: Obar (545 MB) and T (537 MB) exceed the 129 MB L2 every step"),
}
GRAM_ROWS = {"resconv": 32768, "rbm": 8192}  # rows of T = Obar Obar^T ([Re; Im] stacked for ResConv)
# the plain method and the other forms: (name, conv, gram, solve)
PLAIN = {"resconv": ("plain", "fp32", "3xtf32", "fp64"), "rbm": ("plain", "fp32", "3xtf32", "fp64")}
FORMS = {
    "resconv": [("accurate_fp32_conv_3xtf32_gram_mixed_solve", "fp32", "3xtf32", "mixed"),
                ("precision_tf32_conv_tf32_gram_mixed_solve", "tf32", "tf32", "mixed"),
                ("precision_bf16_conv_bf16_gram_mixed_solve", "bf16", "bf16", "mixed")],
    "rbm": [("plain_with_cusolver_fp64_factor", "fp32", "3xtf32", "fp64_lib"),
            ("accurate_3xtf32_gram_mixed_solve", "fp32", "3xtf32", "mixed"),
            ("precision_tf32_gram_mixed_solve", "fp32", "tf32", "mixed")],
}

# DRAM bytes per Gram launch at the bench's shapes (profiles/gram_tc_3xtf32_rows8192_k16640.md):
#   ncu --metrics gpu__time_duration.sum,dram__bytes_read.sum,dram__bytes_write.sum --clock-control none \
#       -k regex:gram_tc -s 2 -c 1 python -m quantax_gb300.kernel_bench gram --mode 3xtf32 --rows 8192 --k 16640 --reps 1
# rbm (8192 x 16640): 5.42 GB read + 0.51 GB written. resconv (32768 x 34944): the capture at 8192 rows x
# 34944 (11.38 + 0.51 GB) scaled by (32768 / 8192)^2, the growth of the tile pairs that re-read the operand.
GRAM_TRAFFIC_BYTES = {("rbm", "3xtf32"): 4.30e9, ("resconv", "3xtf32"): 4 * (32.79e9 + 2.14e9)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


# ---- the CPU restatement (oracle/cpu_vmc.py): whole SR steps, never scaled -------------------------
class CpuWorkload:
    """Initial state of the CPU restatement for a workload at `chains` chains: the same lattice,
    Hamiltonian, model shape and init distribution as the GPU arm, Philox draws from the same
    stream layout."""

    def __init__(self, workload: str, chains: int, seed: int = 1234):
        import numpy as np
        from oracle import lattice, metropolis, rbm as orbm, resconv
        self.workload, self.chains, self.seed, self.step = workload, chains, seed, 0
        if workload == "resconv":
            self.L, self.nb, self.C = 10, 8, 16
            self.params = resconv.init_he(self.nb, self.C, seed=seed)
            self.s = metropolis.init_fixed_up(chains, 100, 50, seed)
            self.nbr = lattice.neighbor_table((10, 10), 1)
            shells = lattice.neighbors((10, 10), [1, 2])
            self.bonds = np.concatenate([shells[0], shells[1]]).astype(np.int64)
            # per bond: diagonal coupling J, off-diagonal element 2 J sign (MSR: sign -1 on J1 bonds)
            self.Jb = np.concatenate([np.tile([1.0, -2.0], (len(shells[0]), 1)),
                                      np.tile([0.5, 1.0], (len(shells[1]), 1))])
            import torch
            from oracle import cpu_vmc
            self.lp = cpu_vmc._resconv_forward(torch.as_tensor(self.params), self.s, self.L, self.nb, self.C)
        else:
            W, b, _ = orbm.init_normal(64, 256, 0.01, seed=seed)
            self.W, self.b = W.astype(np.float64), b.astype(np.float64)
            self.s = metropolis.init_uniform(chains, 64, seed).astype(np.float64)

    def sr_step(self, timings):
        from oracle import cpu_vmc
        if self.workload == "resconv":
            self.params, self.s, self.lp, e = cpu_vmc.resconv_sr_step(
                self.params, self.s, self.lp, self.L, self.nb, self.C, self.nbr, self.bonds, self.Jb, self.seed,
                self.step, 200, timings=timings)
            self.step += 200
        else:
            self.W, self.b, self.s, e = cpu_vmc.sr_step(self.W, self.b, self.s, self.seed, self.step, 64,
                                                        timings=timings)
            self.step += 64
        return e


def _host_threads():
    cores = len(os.sched_getaffinity(0))
    try:
        import threadpoolctl
        threadpoolctl.threadpool_limits(cores)
    except Exception:
        pass
    import torch
    torch.set_num_threads(cores)
    return cores


def time_cpu_steps(workload: str, chains: int, max_steps: int, budget_s: float):
    """Whole SR steps of the CPU restatement: as many as `max_steps`, stopping before a step that
    would end past `budget_s` at the pace of the steps so far (at least one step runs). Returns
    (steps, seconds, per-phase mean seconds, energies)."""
    w = CpuWorkload(workload, chains)
    times, phases, energies = [], {}, []
    while len(times) < max(1, max_steps):
        tm = {}
        t0 = time.perf_counter()
        energies.append(w.sr_step(tm))
        times.append(time.perf_counter() - t0)
        for k, v in tm.items():
            phases[k] = phases.get(k, 0.0) + v
        if sum(times) + sum(times) / len(times) > budget_s:
            break
    n = len(times)
    return n, sum(times), {k: v / n for k, v in phases.items()}, energies


# bounded sample of our line's cpu_baseline: whole steps at a reduced chain count (about 10-30 s)
CPU_SAMPLE_CHAINS = {"resconv": 128, "rbm": 1024}


def cpu_baseline(workload: str):
    cores = _host_threads()
    chains = CPU_SAMPLE_CHAINS[workload]
    w = WORKLOADS[workload]
    n, t, phases, _ = time_cpu_steps(workload, chains, 3, 15.0)
    return {"value": n / t, "unit": UNIT, "cores": cores, "kind": "port", "scaled": False, "chains": chains,
            "steps": n, "samples_per_s": n * chains / t,
            "sample": (f"oracle/cpu_vmc.py: {n} whole SR step(s) of the workload on {chains} of its {w['chains']} "
                       f"chains (sweep, local energies, O, Obar, Gram, FP64 Cholesky solve, update), "
                       f"{t / n:.2f} s per step at that size; not scaled to the full workload"),
            "phases_s": {k: round(v, 4) for k, v in phases.items()}}


def run_reference(args, rank):
    """The reference arm: whole SR steps of the CPU restatement at the full workload on all host
    cores, as many of the requested steps as fit in --ref-budget seconds (at least one); the
    line reports the steps actually timed."""
    if rank != 0:
        return
    cores = _host_threads()
    w = WORKLOADS[args.workload]
    n, t, phases, energies = time_cpu_steps(args.workload, w["chains"], args.steps, args.ref_budget)
    value = n / t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": n, "warmup": 0, "ms_per_step": 1000.0 * t / n, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 model, f64 solve", "data": "synthetic", "config": dict(w),
            "parallelism": f"host cores x{cores}",
            "requested": {"steps": args.steps, "warmup": args.warmup,
                          "note": (f"whole full-size steps only: {n} fit in the {args.ref_budget:.0f} s budget; "
                                   "no warm-up step (each step is minutes of CPU work)")},
            "reference_jax": "unavailable on this box: quantax needs jax/equinox, not installed, no network",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "scaled": False,
                             "sample": (f"oracle/cpu_vmc.py: {n} whole SR step(s) of the full workload "
                                        f"({w['chains']} chains), timed end to end"),
                             "phases_s": {k: round(v, 3) for k, v in phases.items()}},
            "samples_per_s": n * w["chains"] / t, "energies": energies,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def build_workload(qtx, rank, gram, solve, workload="rbm", conv="fp32"):
    from quantax_gb300 import replicas
    import numpy as np
    qtx.set_random_seed(replicas.replica_seed(1234, rank))
    solver = qtx.optimizer.minnorm_shift_eig(ashift=1e-4, precision=solve)
    if workload == "resconv":
        qtx.set_default_dtype(np.complex128)
        qtx.sites.Square(10, Nparticles=(50, 50))
        H = qtx.operator.Heisenberg(J=[1.0, 0.5], n_neighbor=[1, 2], msr=True)
        state = qtx.state.Variational(qtx.model.ResConv(8, 16, out_dtype=np.complex64, conv_precision=conv))
        sampler = qtx.sampler.SpinExchange(state, 16384, thermal_steps=200, sweep_steps=200)
    else:
        qtx.set_default_dtype(np.float64)
        qtx.sites.Chain(64)
        H = qtx.operator.Ising(h=1.0, J=1.0)
        state = qtx.state.Variational(qtx.model.RBM_Dense(256, init_std=0.01))
        sampler = qtx.sampler.LocalFlip(state, 8192, thermal_steps=640, sweep_steps=64)
    opt = qtx.optimizer.SR(state, H, solver=solver, gram=gram)
    return state, sampler, opt


def run_form(args, rank, world, gram, solve, e2e_steps=0, clocks=None, conv="fp32"):
    """Warm-up + timed SR steps of one form; returns timings, phases, energies and, when
    e2e_steps > 0, the end-to-end time of that many steps through the public API."""
    import torch
    import quantax_gb300 as qtx
    from quantax_gb300 import _lib, replicas

    state, sampler, opt = build_workload(qtx, rank, gram, solve, args.workload, conv)
    lr = 1e-2

    def sr_step(ev=None):
        def mark(name):
            if ev is not None:
                e = torch.cuda.Event(enable_timing=True)
                e.record()
                ev.append((name, e))
        samples = sampler.sweep()
        mark("sweep")
        Ebar = opt.get_Ebar(samples)
        mark("eloc")
        Obar = opt.get_Obar(samples)
        mark("obar")
        opt.marks = ev
        step = opt.solve(Obar, Ebar)
        opt.marks = None
        mark("solve")
        state.update(step * lr)
        mark("update")
        return opt.stats

    stats = []
    for _ in range(args.warmup):
        stats.append(sr_step().clone())
    torch.cuda.synchronize()
    if clocks is not None:
        clocks.start()
    replicas.barrier()
    torch.cuda.synchronize()
    launches0 = _lib.launch_count
    start = torch.cuda.Event(enable_timing=True)
    start.record()
    step_events, phase_events = [], []
    for _ in range(args.steps):
        ev = []
        stats.append(sr_step(ev).clone())
        phase_events.append(ev)
        step_events.append(ev[-1][1])
    end = torch.cuda.Event(enable_timing=True)
    end.record()
    torch.cuda.synchronize()
    replicas.barrier()
    clk = clocks.stop() if clocks is not None else None
    launches = _lib.launch_count - launches0
    elapsed = replicas.max_over_ranks(start.elapsed_time(end) / 1000.0, "cuda")
    lat, prev = [], start
    for e in step_events:
        lat.append(prev.elapsed_time(e))
        prev = e
    phases = {}
    for i, ev in enumerate(phase_events):
        prev = start if i == 0 else phase_events[i - 1][-1][1]
        for name, e in ev:
            phases[name] = phases.get(name, 0.0) + prev.elapsed_time(e)
            prev = e
    phases = {k: v / args.steps for k, v in phases.items()}
    if "gram" in phases:
        phases["solve_and_projection"] = phases.pop("solve")
    energies = [float(x[0]) for x in stats[args.warmup:]]
    out = dict(elapsed=elapsed, lat=lat, phases=phases, energies=energies, launches=launches, clocks=clk,
               nparams=state.nparams, fallbacks=opt.solve_fallbacks)

    if args.workload == "resconv" and e2e_steps > 0:
        # the step's dominant kernel on its own: the forward over the chains' current configurations,
        # CUDA events around 10 launches on the stream they run on (after the timed steps)
        packed = sampler.sweep(0).packed
        for _ in range(2):
            state.log_psi_packed(packed)
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record()
        for _ in range(10):
            state.log_psi_packed(packed)
        f1.record()
        torch.cuda.synchronize()
        out["fwd_ms"] = f0.elapsed_time(f1) / 10
        out["fwd_ncfg"] = int(packed.shape[0])

    if e2e_steps > 0:
        # end to end through the public API with host buffers: parameters in from pinned host
        # memory, energy statistics and updated parameters back every step
        host_params = torch.empty(state.nparams, dtype=torch.float32).pin_memory()
        host_params.copy_(state.params.cpu())
        host_out = torch.empty(state.nparams, dtype=torch.float32).pin_memory()
        host_stats = torch.empty(3, dtype=torch.float64).pin_memory()
        torch.cuda.synchronize()
        replicas.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(e2e_steps):
            state.params.copy_(host_params, non_blocking=True)
            state._refresh()
            sr_step()
            host_stats.copy_(opt.stats, non_blocking=True)
            host_out.copy_(state.params, non_blocking=True)
            torch.cuda.current_stream().synchronize()
            host_params.copy_(host_out)
        e1.record()
        torch.cuda.synchronize()
        out["e2e_s"] = replicas.max_over_ranks(e0.elapsed_time(e1) / 1000.0, "cuda")
    return out


def run_serving(args, rank):
    """A seeded Poisson stream of VMC jobs (TFIM chains with RBM_Dense, J1-J2 squares with
    ResConv, sample counts 1024-8192), served with continuous batching on one GPU."""
    from quantax_gb300.serving import JobSpec, VMCServer, poisson_jobs
    specs = poisson_jobs(args.jobs, seed=2024 + rank, steps=args.job_steps)
    # warm-up, untimed: one small job of each kind through its own server, so that loading the
    # solver libraries and first-use module loads do not land in the first timed job's steps
    warm = VMCServer(max_active=2)
    warm.submit(JobSpec("warm_tfim", "tfim", 16, 1024, 3, seed=1))
    warm.submit(JobSpec("warm_j1j2", "j1j2", 4, 1024, 3, seed=2))
    warm.run()
    srv = VMCServer(max_active=8)
    for sp in specs:
        srv.submit(sp)
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    out = srv.run()
    clk = clocks.stop()
    steps = out["steps"]
    ratios = sorted(percentile(j["latencies_ms"], 0.99) / percentile(j["latencies_ms"], 0.5)
                    for j in out["jobs"] if j["latencies_ms"])
    per_job = {"median": ratios[len(ratios) // 2], "max": ratios[-1]} if ratios else None
    if rank == 0:
        line = {"metric": METRIC, "value": steps / out["wall_s"], "unit": UNIT, "n_gpus": 1, "steps": steps,
                "warmup": 2, "warmup_note": "two untimed warm-up jobs (3 SR steps each) through a separate server",
                "ms_per_step": 1000.0 * out["wall_s"] / steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "bf16 conv / bf16 Gram / FP64 solve",
                "data": "synthetic",
                "config": {"workload": f"serving: {args.jobs} Poisson jobs x {args.job_steps} SR steps "
                                       "(config-5 mixture)", "max_active": 8, "conv": specs[0].conv,
                           "gram": specs[0].gram, "solve": specs[0].solve},
                "jobs_per_s": out["jobs_per_s"], "samples_per_s": out["samples_per_s"],
                "p50_step_ms": out["p50_step_ms"], "p99_step_ms": out["p99_step_ms"], "wall_s": out["wall_s"],
                "jobs": [{"name": j["name"], "status": j["status"],
                          "final_energy": j["energies"][-1] if j["energies"] else None,
                          "p50_step_ms": percentile(j["latencies_ms"], 0.5) if j["latencies_ms"] else None,
                          "p99_step_ms": percentile(j["latencies_ms"], 0.99) if j["latencies_ms"] else None}
                         for j in out["jobs"]],
                "per_job_p99_over_p50": per_job,
                "note": ("p50/p99 pool every step of every job, so they span the job sizes of the mixture "
                         "(a 16-site chain to a 10x10 ResConv); per_job_p99_over_p50 is each job's own "
                         "step-latency spread while it shares the GPU with the others"),
                "clocks": clk}
        print(json.dumps(line), flush=True)


def run_trajectory(args, rank):
    """Energy trajectories of the plain path and the precision forms from identical initial
    parameters and seeds: J1-J2 (J2 = 0.5, MSR) on the 10x10 square, ResConv(8 blocks, 16
    channels, complex output), SpinExchange with 200 proposals per sweep, MinSR with diagonal
    shift 1e-4, learning rate 1e-2. The chain count is reduced from 16384 to --chains (the
    FP64 plain path factorises a 2Ns x 2Ns matrix every step). Reports every form's energies,
    the mean and standard error over the last quarter, and the relative difference of that
    mean to the plain path's."""
    import numpy as np
    import torch
    import quantax_gb300 as qtx
    forms = [tuple(f.split(":")) for f in args.forms.split(",")]
    out = {}
    for name, conv, gram, solve in forms:
        qtx.set_random_seed(4321)
        qtx.set_default_dtype(np.complex128)
        qtx.sites.Square(10, Nparticles=(50, 50))
        H = qtx.operator.Heisenberg(J=[1.0, 0.5], n_neighbor=[1, 2], msr=True)
        state = qtx.state.Variational(qtx.model.ResConv(8, 16, out_dtype=np.complex64, conv_precision=conv))
        sampler = qtx.sampler.SpinExchange(state, args.chains, thermal_steps=200, sweep_steps=200)
        if solve == "pinv":  # config 4's FP64 pseudo-inverse: eigendecomposition with rtol 1e-12
            solver = qtx.optimizer.minnorm_pinv_eig(rtol=1e-12)
        elif solve == "pinv_atol":  # the same with the soft cutoff also at the shift's scale, 1e-4
            solver = qtx.optimizer.minnorm_pinv_eig(rtol=1e-12, atol=1e-4)
        else:
            solver = qtx.optimizer.minnorm_shift_eig(ashift=1e-4, precision=solve)
        opt = qtx.optimizer.SR(state, H, solver=solver, gram=gram)
        stats = []
        skipped = 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step = opt.get_step(sampler.sweep())
            skipped += int(not bool(torch.isfinite(step).all()))
            state.update(step * 1e-2)
            stats.append(opt.stats.clone())
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        e = np.array([float(x[0]) for x in stats])
        tail = e[-max(1, len(e) // 4):]
        out[name] = {"conv": conv, "gram": gram, "solve": solve, "s_per_step": wall / len(e),
                     "fp64_fallbacks": opt.solve_fallbacks, "nonfinite_steps": skipped,
                     "energies": [round(float(v), 6) for v in e], "tail_mean": float(tail.mean()),
                     "tail_stderr": float(tail.std(ddof=1) / np.sqrt(len(tail))) if len(tail) > 1 else None}
        qtx.set_default_dtype(np.float64)
    ref = out[forms[0][0]]["tail_mean"]
    for name in out:
        out[name]["tail_rel_diff_vs_plain"] = abs(out[name]["tail_mean"] - ref) / abs(ref)
    if rank == 0:
        print(json.dumps({"workload": "trajectory: J1-J2 10x10, ResConv(8, 16) complex, MinSR shift 1e-4",
                          "chains": args.chains, "steps": args.steps, "forms": out}), flush=True)


# ED ground energies of the 4x4 Heisenberg and J1-J2 (J2 = 0.5) models (MSR) and the reference's
# trained, projected ResConv(2 blocks, 8 channels) on them (tutorials/J1J2.ipynb:90, :331,
# :374, :562). The Heisenberg figure is the projection of the unsymmetrised 200-step model
# (the notebook's second loop updates the unprojected state); the J1-J2 one follows 200
# steps of the projected state.
TUTORIALS = {
    "heisenberg_tutorial": dict(J=[1.0], n_neighbor=[1], sinhp1=False, ed=-44.91393283371544,
                                reference={"energy": -44.91365075323898, "rel_err": 6.280467076974902e-06,
                                           "fidelity": 0.9999925315217684,
                                           "state": "projected_after_unsymmetrised_training"}),
    "j1j2_tutorial": dict(J=[1.0, 0.5], n_neighbor=[1, 2], sinhp1=True, ed=-33.831693405579394,
                          reference={"energy": -33.782434819834265, "rel_err": 0.001455989363423509,
                                     "fidelity": 0.9971699670582732, "state": "projected_training"}),
}


def exact_energy(qtx, state, H):
    """<psi|H|psi> / <psi|psi> summed over every Sz = 0 configuration of the 4x4 lattice:
    psi and E_loc from the device kernels, weights |psi|^2 (no sampling)."""
    import numpy as np
    import torch
    from quantax_gb300.sampler import Samples
    from quantax_gb300.state import pack_spins
    n = state.Nmodes
    codes = np.arange(1 << n, dtype=np.int64)
    pop = np.zeros_like(codes)
    for i in range(n):
        pop += (codes >> i) & 1
    codes = codes[pop == n // 2]
    spins = (((codes[:, None] >> np.arange(n)) & 1) * 2 - 1).astype(np.int8)
    packed = pack_spins(spins, n)
    lp = state.log_psi_packed(packed)
    lpr = lp.real if lp.is_complex() else lp
    samples = Samples(packed, lp, n, None)
    E = H.Oloc(state, samples)
    E = E.real if E.is_complex() else E
    w = torch.exp(2.0 * (lpr.double() - lpr.max().double()))
    live = (w > 0) & torch.isfinite(E)
    return float((w[live] * E[live]).sum() / w[live].sum()), int(codes.size)


def run_tutorial(args, rank):
    """The reference's 4x4 notebook (tutorials/J1J2.ipynb: cells 1-19 Heisenberg with
    exp_by_scale, cells 21-30 J1-J2 with sinhp1_by_scale): ResConv(2 blocks, 8 channels)
    trained 200 SR steps (lr 0.01, 1024 SpinExchange samples, default pinv solver) without
    symmetry, then projected on Rotation(pi/2) @ Flip() @ SpinInverse(); and 200 more steps of
    the projected state. Energies are exact sums over the 12870-state sector; times are CUDA
    events around each phase."""
    import numpy as np
    import torch
    import quantax_gb300 as qtx
    from quantax_gb300.symmetry import Flip, Rotation, SpinInverse
    tut = TUTORIALS[args.workload]
    qtx.set_random_seed(args.seed)
    qtx.set_default_dtype(np.float64)
    qtx.sites.Square(4, Nparticles=(8, 8))
    H = qtx.operator.Heisenberg(J=tut["J"], n_neighbor=tut["n_neighbor"], msr=True)
    model = qtx.model.ResConv(2, 8, final_activation=qtx.nn.sinhp1_by_scale if tut["sinhp1"] else None)

    def train(state, steps):
        sampler = qtx.sampler.SpinExchange(state, 1024)
        opt = qtx.optimizer.SR(state, H)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        energies = []
        for _ in range(steps):
            samples = sampler.sweep()
            step = opt.get_step(samples)
            state.update(step * 0.01)
            energies.append(opt.stats)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1000.0, [float(x[0]) for x in energies]

    state = qtx.state.Variational(model)
    t1, en1 = train(state, args.tutorial_steps)
    e_plain, dim = exact_energy(qtx, state, H)
    symm = Rotation(np.pi / 2) @ Flip() @ SpinInverse()
    symm_state = qtx.state.Variational(model, symm=symm)
    symm_state.set_params(state.params.cpu())
    e_proj, _ = exact_energy(qtx, symm_state, H)
    t2, en2 = train(symm_state, args.tutorial_steps)
    e_proj2, _ = exact_energy(qtx, symm_state, H)
    ed = tut["ed"]
    rel = lambda e: abs((e - ed) / ed)
    line = {
        "metric": "relative energy error of the projected state",
        "workload": args.workload.replace("_tutorial", "") + "_square4_resconv2x8_tutorial",
        "final_activation": "sinhp1_by_scale" if tut["sinhp1"] else "exp_by_scale",
        "ed_energy": ed, "sector_dim": dim, "seed": args.seed, "steps_per_phase": args.tutorial_steps,
        "reference": tut["reference"],
        "unsymmetrised_training": {"steps_per_s": args.tutorial_steps / t1, "exact_energy": e_plain,
                                   "rel_err": rel(e_plain), "mc_energy_last10": float(np.mean(en1[-10:]))},
        "projected_after_unsymmetrised_training": {"exact_energy": e_proj, "rel_err": rel(e_proj),
                                                   "nsymm": symm.nsymm},
        "projected_training": {"steps_per_s": args.tutorial_steps / t2, "exact_energy": e_proj2,
                               "rel_err": rel(e_proj2), "mc_energy_last10": float(np.mean(en2[-10:]))},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# examples/RBM.ipynb: 10 x 10 Heisenberg (MSR), QMC energy and the reference's relative error of
# the mean of its last 100 SR steps (cells 3-5)
RBM_EXAMPLE_E_QMC = -268.62107
RBM_EXAMPLE_REFERENCE_REL_ERR = 0.0009721019350138251


def run_rbm_example(args, rank):
    """The reference's examples/RBM.ipynb: RBM_Conv(16) on the 10 x 10 Heisenberg model (MSR),
    8192 SpinExchange samples, SR with lstsq_pinv_eig(rtol=1e-9) (FP64 Gram, the cut-off lies
    below FP32 resolution), lr 2e-3; the energy is the mean of the last 100 steps' MC energies,
    against the QMC value. Times are CUDA events around the training loop."""
    import numpy as np
    import torch
    import quantax_gb300 as qtx
    qtx.set_random_seed(args.seed)
    qtx.set_default_dtype(np.float64)
    qtx.sites.Square(10, Nparticles=(50, 50))
    H = qtx.operator.Heisenberg(msr=True)
    state = qtx.state.Variational(qtx.model.RBM_Conv(16))
    sampler = qtx.sampler.SpinExchange(state, 8192)
    opt = qtx.optimizer.SR(state, H, solver=qtx.optimizer.lstsq_pinv_eig(rtol=1e-9), gram="fp64")
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    stats = []
    for _ in range(args.example_steps):
        samples = sampler.sweep()
        step = opt.get_step(samples)
        state.update(step * 2e-3)
        stats.append(opt.stats.clone())
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1000.0
    energies = np.array([float(x[0]) for x in stats])
    tail = energies[-min(100, len(energies)):]
    E = float(tail.mean())
    line = {"metric": "relative energy error vs QMC", "workload": "heisenberg_square10_rbm_conv16_example",
            "seed": args.seed, "steps": args.example_steps, "steps_per_s": args.example_steps / t,
            "ms_per_step": 1000.0 * t / args.example_steps, "energy_last100_mean": E,
            "rel_err": (E - RBM_EXAMPLE_E_QMC) / abs(RBM_EXAMPLE_E_QMC), "e_qmc": RBM_EXAMPLE_E_QMC,
            "reference_rel_err": RBM_EXAMPLE_REFERENCE_REL_ERR,
            "energy_every_100": [float(energies[i]) for i in range(0, len(energies), 100)],
            "solve_fallbacks": opt.solve_fallbacks}
    if rank == 0:
        print(json.dumps(line), flush=True)


def percentile(lat, q):
    s = sorted(lat)
    return s[min(len(s) - 1, int(round(q * (len(s) - 1))))]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="resconv",
                    choices=["resconv", "rbm", "serving", "trajectory", "heisenberg_tutorial", "j1j2_tutorial",
                             "rbm_example"],
                    help="resconv: J1-J2 10x10 with ResConv (the default line); rbm: chain-64 TFIM with RBM 256; "
                         "serving: a Poisson stream of jobs through quantax_gb300.serving")
    ap.add_argument("--gram", default=None, choices=["fp32", "tf32", "bf16", "3xtf32"],
                    help="Gram of the plain method (default split-TF32 on the tensor cores, FP32-class: "
                         "accumulation error 6.6e-6 against 8.2e-5 for fp32 on the CUDA cores)")
    ap.add_argument("--solve", default=None, choices=["fp64", "fp64_lib", "mixed"],
                    help="solve of the plain method: fp64 (qgx_cholesky), fp64_lib (cuSOLVER Xpotrf), mixed")
    ap.add_argument("--conv", default=None, choices=["fp32", "tf32", "bf16"],
                    help="resconv: arithmetic of the plain method's convolutions")
    ap.add_argument("--e2e-steps", type=int, default=None,
                    help="steps of the end-to-end (host buffers) measurement; default min(steps, 5)")
    ap.add_argument("--ref-budget", type=float, default=300.0,
                    help="--impl reference: seconds of whole CPU steps to time (at least one step runs)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the other forms")
    ap.add_argument("--tutorial-steps", type=int, default=200, help="*_tutorial: SR steps per phase")
    ap.add_argument("--seed", type=int, default=0, help="*_tutorial, rbm_example: random seed")
    ap.add_argument("--example-steps", type=int, default=1000, help="rbm_example: SR steps")
    ap.add_argument("--jobs", type=int, default=8, help="serving: number of jobs in the stream")
    ap.add_argument("--chains", type=int, default=2048, help="trajectory: Markov chains (samples per step)")
    ap.add_argument("--forms", default="plain:fp32:3xtf32:fp64,precision_bf16:bf16:bf16:mixed,"
                                       "precision_tf32:tf32:tf32:mixed,precision_bf16_pinv:bf16:bf16:pinv",
                    help="trajectory: comma-separated name:conv:gram:solve (solve fp64, fp64_lib, mixed, pinv: "
                         "the FP64 pseudo-inverse with rtol 1e-12, or pinv_atol: the same with atol 1e-4); "
                         "the first is the reference run")
    ap.add_argument("--job-steps", type=int, default=50, help="serving: SR steps per job")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if args.workload not in WORKLOADS:
            raise SystemExit("--impl reference times the resconv and rbm workloads")
        run_reference(args, rank)
        return

    import torch
    import torch.distributed as dist

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from quantax_gb300 import _build
    _build.build()

    if args.workload == "serving":
        run_serving(args, rank)
        return
    if args.workload == "trajectory":
        run_trajectory(args, rank)
        return
    if args.workload in TUTORIALS:
        run_tutorial(args, rank)
        return
    if args.workload == "rbm_example":
        run_rbm_example(args, rank)
        return

    wl = args.workload
    _, conv0, gram0, solve0 = PLAIN[wl]
    conv, gram, solve = args.conv or conv0, args.gram or gram0, args.solve or solve0
    e2e_steps = min(args.steps, 5) if args.e2e_steps is None else args.e2e_steps
    plain = run_form(args, rank, world, gram, solve, e2e_steps=e2e_steps,
                     clocks=Clocks(local) if rank == 0 else None, conv=conv)
    chains = WORKLOADS[wl]["chains"]
    forms = {}
    if not args.no_forms:
        for name, fconv, fgram, fsolve in FORMS[wl]:
            prec = run_form(args, rank, world, fgram, fsolve, conv=fconv)
            de = [abs(a - b) / abs(b) for a, b in zip(prec["energies"], plain["energies"])]
            forms[name] = {
                "value": world * args.steps / prec["elapsed"], "unit": UNIT,
                "method": {"conv": fconv, "gram": fgram, "solve": fsolve},
                "ms_per_step": 1000.0 * prec["elapsed"] / args.steps,
                "samples_per_s": world * args.steps * chains / prec["elapsed"],
                "p50_step_ms": percentile(prec["lat"], 0.5), "p99_step_ms": percentile(prec["lat"], 0.99),
                "phases_ms": {k: round(v, 4) for k, v in prec["phases"].items()},
                "speedup_vs_plain": plain["elapsed"] / prec["elapsed"],
                "fp64_fallbacks": prec["fallbacks"],
                "energies": [round(e, 6) for e in prec["energies"]],
                "energy_rel_diff_vs_plain_max": max(de), "energy_rel_diff_vs_plain_last": de[-1]}

    if rank == 0:
        hbm, bf16, src = peaks()
        npar = plain["nparams"]
        ns = GRAM_ROWS[wl]
        phases = plain["phases"]
        gram_flop = 2.0 * ns * ns * npar  # algorithmic: 2 Ns^2 Np (the symmetric half is not counted as saved)
        t_gram = phases.get("gram", float("nan")) / 1000.0
        achieved = gram_flop / t_gram / 1e12
        rate = {"bf16": 1.0, "tf32": 0.5, "3xtf32": 0.5 / 3.0, "fp32": None}[gram]
        roof = {"kernel": f"gram_tc_kernel ({gram}, T = Obar Obar^T)", "bound": "tensor", "achieved": achieved,
                "peak": bf16, "unit": "TFLOP/s", "frac": achieved / bf16,
                "peak_source": f"bf16 dense burst, {src} (MEASURED_PEAKS.json)",
                "mode_peak": None if rate is None else bf16 * rate,
                "frac_of_mode_peak": None if rate is None else achieved / (bf16 * rate),
                "traffic": GRAM_TRAFFIC_BYTES.get((wl, gram)),
                "traffic_unit": ("bytes per launch (ncu dram__bytes_read + write"
                                 + (", the 16384-row capture scaled by (32768 / 16384)^2; "
                                    "profiles/gram_tc_3xtf32_rows8192_k16640.md)" if wl == "resconv"
                                    else "; profiles/gram_tc_3xtf32_rows8192_k16640.md)")),
                "algorithmic": (f"2 Ns^2 Np = {gram_flop:.3e} FLOP per launch (Ns = {ns} rows, Np = {npar}); operand "
                                f"{ns * npar * 4:.3e} B read, T {ns * ns * 8:.3e} B written"),
                "duration": "CUDA events around the Gram phase (one launch) of every timed step, mean",
                "note": ("split-TF32: each product is hi*hi + hi*lo + lo*hi, so its mode peak is a third of the TF32 "
                         "rate" if gram == "3xtf32" else "")}
        roof_fwd = None
        if "fwd_ms" in plain and conv == "fp32":
            L, nb, ch = 10, 8, 16
            flop = 2.0 * L * L * 9 * ch * (1 + (2 * nb - 1) * ch)  # 6.94e6 per forward
            ach = flop * plain["fwd_ncfg"] / (plain["fwd_ms"] / 1000.0) / 1e12
            fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
            roof_fwd = {"kernel": "rc_forward_kernel (ResConv forward, FP32 on the CUDA cores, blocked site order)",
                        "bound": "fp32", "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s",
                        "frac": ach / fp32_peak,
                        "peak_source": ("nominal FP32 FMA rate, 152 SMs x 128 lanes x 2 FLOP x 2.07 GHz "
                                        "(MEASURED_PEAKS.json holds no FP32 figure)"),
                        "algorithmic": (f"{flop:.4e} FLOP per forward x {plain['fwd_ncfg']} configurations per "
                                        "launch"),
                        "duration": (f"{plain['fwd_ms']:.4f} ms per launch: CUDA events around 10 launches over "
                                     "the step's chains, after the timed steps"),
                        "note": ("the plain step's largest kernel (about half its device time: sweep proposals and "
                                 "local energies, profiles/launches_c3_plain_step.md); `roofline` above is the "
                                 "tensor-core Gram")}
        elapsed = plain["elapsed"]
        target = None
        if forms:
            best = max(forms, key=lambda k: forms[k]["speedup_vs_plain"])
            target = {"form": best, "speedup_vs_plain": forms[best]["speedup_vs_plain"],
                      "energy_rel_diff_vs_plain_max": forms[best]["energy_rel_diff_vs_plain_max"],
                      "p99_step_ms": forms[best]["p99_step_ms"],
                      "note": (f"over {args.steps} steps from identical initial parameters and seeds; the 200-step "
                               "trajectory comparison is `--workload trajectory`")}
        line = {
            "metric": METRIC, "value": world * args.steps / elapsed, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * elapsed / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 solve)",
            "data": "synthetic", "config": dict(WORKLOADS[wl]), "parallelism": f"replicas x{world}",
            "method": {"conv": conv if wl == "resconv" else None, "gram": gram, "solve": solve},
            "samples_per_s": world * args.steps * chains / elapsed, "p50_step_ms": percentile(plain["lat"], 0.5),
            "p99_step_ms": percentile(plain["lat"], 0.99),
            "phases_ms": {k: round(v, 4) for k, v in phases.items()}, "energy": plain["energies"][-1],
            "energies": [round(e, 6) for e in plain["energies"]],
            "e2e": {"value": world * e2e_steps / plain["e2e_s"], "unit": UNIT, "steps": e2e_steps,
                    "h2d_bytes_per_step": npar * 4, "d2h_bytes_per_step": npar * 4 + 24},
            "gpu_launches": plain["launches"], "roofline": roof, "roofline_dominant": roof_fwd,
            "clocks": plain["clocks"], "forms": forms,
            "target": target,
        }
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(wl)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
