"""The chain-sharded MinSR step (quantax_gb300.sharded) as two gloo ranks on CPU: each rank holds
half of the samples, exchanges the statistics, the Obar row blocks and T's block rows, and
must produce the single-process step of the oracle (minnorm_shift_eig on all samples,
quantax/optimizer/solver.py:50-62 with sr.py:76-113) to 1e-10 relative."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from oracle import sr as osr

NS, NP = 64, 150


def _problem(complex_out, seed=7):
    rng = np.random.default_rng(seed)
    O = rng.normal(size=(NS, NP)) + (1j * rng.normal(size=(NS, NP)) if complex_out else 0)
    E = rng.normal(size=NS) - 30.0 + (1j * 0.1 * rng.normal(size=NS) if complex_out else 0)
    return O, E


def _oracle_step(O, E, complex_out):
    eb, energy, var = osr.ebar(E)
    x = osr.solve(osr.obar(O), eb, lambda A, b: osr.minnorm_shift(A, b, rshift=1e-12, ashift=1e-4),
                  complex_out=complex_out)
    return x, energy, var


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, complex_out, out):
    import torch.distributed as dist
    from quantax_gb300.sharded import ShardedMinSR
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        O, E = _problem(complex_out)
        rows = slice(rank * NS // world, (rank + 1) * NS // world)
        opt = ShardedMinSR(rshift=1e-12, ashift=1e-4)
        x = opt.step(torch.as_tensor(O[rows]), torch.as_tensor(E[rows]))
        out.put((rank, x.numpy(), opt.energy, opt.VarE))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("complex_out", [False, True])
def test_two_gloo_ranks_equal_single_process_step(complex_out):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, complex_out, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted((q.get(timeout=10) for _ in range(2)), key=lambda t: t[0])
    O, E = _problem(complex_out)
    x_ref, energy, var = _oracle_step(O, E, complex_out)
    for _, x, e, v in res:
        assert np.linalg.norm(x - x_ref) <= 1e-10 * np.linalg.norm(x_ref)
        assert e == pytest.approx(energy, rel=1e-12) and v == pytest.approx(var, rel=1e-10)
    assert np.array_equal(res[0][1], res[1][1])  # every rank applies the same step


def test_single_process_and_divisibility():
    from quantax_gb300.sharded import ShardedMinSR, check_divisible
    O, E = _problem(True, seed=3)
    x = ShardedMinSR().step(torch.as_tensor(O), torch.as_tensor(E)).numpy()
    x_ref, _, _ = _oracle_step(O, E, True)
    assert np.linalg.norm(x - x_ref) <= 1e-10 * np.linalg.norm(x_ref)
    with pytest.raises(ValueError, match="split evenly"):
        check_divisible(10, 3)
