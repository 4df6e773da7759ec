"""Serving form: jobs of different kinds and sizes served concurrently give the same
results as when each runs alone (stated tolerance: 1e-12 relative on every step's energy;
the kernels use fixed reduction orders, so the results are expected to be identical)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _specs():
    from quantax_gb300.serving import JobSpec
    return [
        JobSpec("tfim_a", "tfim", 16, 512, 4, seed=11, h=0.8, alpha=2),
        JobSpec("j1j2_b", "j1j2", 4, 256, 3, seed=12, J2=0.3, blocks=2, channels=8),
        JobSpec("tfim_c", "tfim", 32, 1024, 3, seed=13, h=1.2, alpha=1, arrival=0.05),
    ]


def test_serving_alone_equals_mixed(cuda):
    from quantax_gb300.serving import VMCServer
    alone = {}
    for spec in _specs():
        srv = VMCServer(max_active=1)
        srv.submit(spec)
        out = srv.run()
        alone[spec.name] = out["jobs"][0]["energies"]
    srv = VMCServer(max_active=3)
    for spec in _specs():
        srv.submit(spec)
    out = srv.run()
    assert len(out["jobs"]) == 3 and out["p99_step_ms"] is not None
    for job in out["jobs"]:
        a = np.array(alone[job["name"]])
        m = np.array(job["energies"])
        assert len(a) == len(m)
        assert np.all(np.abs(a - m) <= 1e-12 * np.abs(a)), (job["name"], a, m)


def test_serving_admission_by_budget(cuda):
    from quantax_gb300.serving import VMCServer
    specs = _specs()
    biggest = max(s.hbm_bytes() for s in specs)
    srv = VMCServer(hbm_budget_bytes=biggest + 1, max_active=3)  # only one job fits at a time
    for s in specs:
        srv.submit(s)
    out = srv.run()
    assert sorted(j["name"] for j in out["jobs"]) == sorted(s.name for s in specs)
    with pytest.raises(ValueError):
        VMCServer(hbm_budget_bytes=1).submit(specs[0])
