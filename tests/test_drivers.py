"""The time-stepping drivers (quantax/optimizer/driver.py:9-104) on the CPU with stand-ins for
the sampler, the optimizer and the state: the order of sweeps, solves and updates, and the
adaptive step-length rule."""
import numpy as np
import torch

from quantax_gb300.optimizer import AdaptiveHeunEvolution, Euler


class _State:
    def __init__(self):
        self.updates = []

    def update(self, step):
        self.updates.append(step.clone())


class _Sampler:
    def __init__(self):
        self.n = 0

    def sweep(self):
        self.n += 1
        return self.n


class _TDVP:
    """get_step(samples) = a fixed vector per sweep; S = diag(s)."""

    def __init__(self, steps, s_diag):
        self.steps = steps
        self.S = torch.diag(torch.as_tensor(s_diag, dtype=torch.float64))
        self.calls = []
        self.energy, self.VarE = -1.5, 0.25

    def get_step(self, samples):
        self.calls.append(("step", samples))
        return self.steps[samples - 1]

    def get_SF(self, samples):
        self.calls.append(("SF", samples))
        return self.S.clone(), torch.zeros(self.S.shape[0], dtype=torch.float64)

    def solve(self, S, F):
        self.calls.append(("solve",))
        return self.steps[4]


def test_euler_driver():
    st, sp = _State(), _Sampler()
    steps = [torch.tensor([1.0, 2.0], dtype=torch.float64), torch.tensor([3.0, 4.0], dtype=torch.float64)]
    opt = _TDVP(steps + steps + steps, [1.0, 1.0])
    d = Euler(st, sp, opt, 0.1)
    d.step()
    d.step()
    assert [u.tolist() for u in st.updates] == [(0.1 * steps[0]).tolist(), (0.1 * steps[1]).tolist()]
    np.testing.assert_allclose(d.energy.time, [0.1, 0.2])
    np.testing.assert_array_equal(d.energy.data, [-1.5, -1.5])
    np.testing.assert_array_equal(d.VarE.data, [0.25, 0.25])


def test_adaptive_heun_sequence_and_step_length():
    rng = np.random.default_rng(0)
    steps = [torch.as_tensor(rng.normal(size=3)) for _ in range(5)]
    si, sf, sm, smm, sff = steps
    st, sp = _State(), _Sampler()
    s_diag = [2.0, 0.5, 1.0]
    tdvp = _TDVP(steps, s_diag)
    dt = 2e-3
    d = AdaptiveHeunEvolution(st, sp, tdvp, step_length=dt, integ_threshold=1e-3)
    d.step()
    assert tdvp.calls == [("step", 1), ("step", 2), ("step", 3), ("step", 4), ("SF", 5), ("solve",)]
    want = [dt * si, -dt / 2 * si, dt / 4 * (sm - si), dt / 2 * smm, dt / 4 * (sff - smm)]
    for u, w in zip(st.updates, want):
        torch.testing.assert_close(u, w, rtol=0, atol=0)
    # the state ends at theta - dt (si + sm + smm + sff) / 4 (the two half steps)
    torch.testing.assert_close(sum(st.updates), dt * (si + sm + smm + sff) / 4, rtol=1e-14, atol=1e-17)
    diff = ((si + sf) / 2 - (si + sm + smm + sff) / 4).numpy()
    err = np.sqrt(diff @ np.diag(s_diag) @ diff) * dt
    new_dt = float(np.clip(dt * np.clip((1e-3 / err) ** (1 / 3), 0.2, 2), 1e-4, 1e-2))
    assert d.step_length == new_dt and d.time == new_dt
    np.testing.assert_array_equal(d.step_size.data, [new_dt])
    np.testing.assert_array_equal(d.step_size.time, [new_dt])


def test_adaptive_heun_limits():
    """A zero error estimate doubles the step (ratio clipped at 2), a huge one cuts it to a
    fifth, and the length stays within [1e-4, 1e-2]."""
    same = [torch.ones(2, dtype=torch.float64)] * 5
    d = AdaptiveHeunEvolution(_State(), _Sampler(), _TDVP(same, [1.0, 1.0]), step_length=2e-3)
    d.step()
    assert d.step_length == 4e-3
    big = [torch.full((2,), x, dtype=torch.float64) for x in (0.0, 1e6, 0.0, 0.0, 0.0)]
    d = AdaptiveHeunEvolution(_State(), _Sampler(), _TDVP(big, [1.0, 1.0]), step_length=2e-4)
    d.step()
    assert d.step_length == 1e-4  # 2e-4 / 5 clipped up to the lower limit
