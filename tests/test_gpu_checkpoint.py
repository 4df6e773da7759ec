"""Variational.save / Variational(model, param_file) through the reference's checkpoint
format, as the J1-J2 notebook uses them (state saved, then reloaded under a symmetry)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_state_checkpoint_round_trip(cuda, tmp_path):
    import quantax_gb300 as qtx
    from quantax_gb300.symmetry import Flip, Rotation, SpinInverse
    qtx.set_random_seed(2)
    qtx.set_default_dtype(np.float64)
    qtx.sites.Square(4, Nparticles=(8, 8))
    model = qtx.model.ResConv(2, 8)
    state = qtx.state.Variational(model)
    state.update(torch.linspace(-1e-2, 1e-2, state.nparams, dtype=torch.float64).cuda())
    f = tmp_path / "model.eqx"
    state.save(f)
    again = qtx.state.Variational(model, f)
    assert torch.equal(again.params, state.params)
    symm_state = qtx.state.Variational(model, f, Rotation(np.pi / 2) @ Flip() @ SpinInverse())
    assert torch.equal(symm_state.params, state.params)
    s = np.array([[1, -1] * 8, [1] * 8 + [-1] * 8])
    torch.testing.assert_close(again.log_psi(s), state.log_psi(s))
