"""Batched RBM sweeps and local energies (qgx_rbm_sweep_batched / qgx_rbm_eloc_batched), the
shared launches of the serving loop's RBM jobs, against each job's own sweep() and Oloc():
chains, log psi, accept counts and local energies must be equal bit for bit, since every job
runs the same device function on its own chains, Philox streams and table."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

# (L, alpha, samples): hidden-unit widths 16 .. 512 (three width classes, tables staged in
# shared memory and read from global memory), ragged sample counts
SHAPES = [(16, 2, 300), (32, 1, 1024), (64, 4, 512), (128, 4, 257), (8, 2, 64)]


def _pair(L, alpha, ns, seed):
    """Two identical TFIM jobs (same seed): one for the single calls, one for the batch."""
    from quantax_gb300.serving import Job, JobSpec
    spec = JobSpec(f"tfim{L}", "tfim", L, ns, 3, seed=seed, h=0.9, alpha=alpha)
    return Job(spec, torch.cuda.current_stream()), Job(spec, torch.cuda.current_stream())


def test_batched_sweeps_and_local_energies_equal_single_calls(cuda):
    from quantax_gb300.operator import Operator
    from quantax_gb300.sampler import Metropolis
    pairs = [_pair(L, a, ns, 40 + k) for k, (L, a, ns) in enumerate(SHAPES)]
    for rnd in range(3):  # three sweeps: the step counters advance alike
        single = [a.sampler.sweep() for a, _ in pairs]
        batched = Metropolis.sweep_batched([b.sampler for _, b in pairs])
        e_single = [a.opt.hamiltonian.Oloc(a.state, s) for (a, _), s in zip(pairs, single)]
        e_batched = Operator.Oloc_batched([(b.opt.hamiltonian, b.state, s) for (_, b), s in zip(pairs, batched)])
        torch.cuda.synchronize()
        for (a, b), s1, s2, e1, e2 in zip(pairs, single, batched, e_single, e_batched):
            assert torch.equal(s1.packed, s2.packed), (a.spec.name, rnd)
            assert torch.equal(s1.log_psi, s2.log_psi), (a.spec.name, rnd)
            assert torch.equal(a.sampler.accepts, b.sampler.accepts), (a.spec.name, rnd)
            assert torch.equal(e1, e2), (a.spec.name, rnd)
        # move the parameters between sweeps, identically in both copies
        for a, b in pairs:
            for job in (a, b):
                job.state.update(torch.full((job.state.nparams,), 1e-3, dtype=torch.float64, device="cuda"))


def test_batched_launch_counts(cuda):
    """Jobs of one class share a launch: the five LocalFlip jobs' hidden units pad to 128, 128,
    256, 512 and 128 (three width classes; a table too large for shared memory could split a
    class), so the batch makes three or four launches for five jobs."""
    import ctypes as C
    from quantax_gb300 import _lib
    jobs = [_pair(L, a, ns, 60 + k)[0] for k, (L, a, ns) in enumerate(SHAPES)]
    descs = [j.sampler._batch_job(j.sampler._sweep_steps) for j in jobs]
    arr = (_lib.RbmSweepJob * len(descs))(*descs)
    launches = C.c_int32(-1)
    _lib.call("qgx_rbm_sweep_batched", arr, len(descs), C.byref(launches), _lib.stream_ptr())
    torch.cuda.synchronize()
    assert 3 <= launches.value <= 4


def test_batched_sweep_arguments(cuda):
    import ctypes as C
    from quantax_gb300 import _lib
    lib = _lib.lib()
    too_many = (_lib.RbmSweepJob * (_lib.RBM_BATCH_MAX_JOBS + 1))()
    assert lib.qgx_rbm_sweep_batched(too_many, _lib.RBM_BATCH_MAX_JOBS + 1, None, None) == _lib.QGX_ERR_ARG
    bad = (_lib.RbmSweepJob * 1)()
    bad[0].n, bad[0].m, bad[0].ns, bad[0].proposal = 16, 32, 8, 99
    assert lib.qgx_rbm_sweep_batched(bad, 1, None, None) == _lib.QGX_ERR_ARG
    assert lib.qgx_rbm_sweep_batched(None, 0, None, None) == _lib.QGX_OK


def test_serving_batched_equals_unbatched(cuda):
    """The server's batched front (RBM jobs' sweeps and local energies in shared launches)
    changes no job's energies: equal to the unbatched server's, step by step."""
    from quantax_gb300.serving import JobSpec, VMCServer
    specs = lambda: [JobSpec("t16", "tfim", 16, 512, 4, seed=5, h=0.7, alpha=2),
                     JobSpec("t32", "tfim", 32, 1024, 4, seed=6, h=1.1, alpha=4),
                     JobSpec("t64", "tfim", 64, 256, 4, seed=7, h=1.0, alpha=1),
                     JobSpec("j4", "j1j2", 4, 256, 4, seed=8, J2=0.4, blocks=2, channels=8)]
    runs = {}
    for batch in (False, True):
        srv = VMCServer(max_active=4, batch=batch)
        for sp in specs():
            srv.submit(sp)
        out = srv.run()
        runs[batch] = {j["name"]: np.array(j["energies"]) for j in out["jobs"]}
        if batch:
            assert srv.batched_rounds >= 4
    for name, e in runs[False].items():
        assert np.array_equal(e, runs[True][name]), name
