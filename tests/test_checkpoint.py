"""Checkpoints in the reference's format (equinox leaf records, quantax_gb300.checkpoint).

equinox is absent here, so the reference cannot write a file in this container: the
reference-side files are synthesised record by record from its leaf order (the dataclass
fields of quantax/model/shallow_nets.py:35-78, quantax/model/conv_nets.py:26-183 and
quantax/nn/modules.py:9-37, equinox Conv / Linear weight and bias shapes). Parity with a file
written by quantax itself is unpinned."""
import io

import numpy as np
import pytest

from quantax_gb300 import checkpoint as ck


def _records(buf):
    buf.seek(0)
    out = []
    while True:
        try:
            out.append(np.load(buf, allow_pickle=False))
        except (EOFError, ValueError):
            return out


@pytest.fixture
def square4():
    import quantax_gb300 as qtx
    qtx.set_default_dtype(np.float64)
    qtx.sites.Square(4, Nparticles=(8, 8))
    return qtx


def test_resconv_record_sequence(square4):
    """ResConv(2 blocks, 8 channels): conv1.weight, conv1.bias (C, 1, 1), conv2.weight,
    conv2.bias for block 0, the same without conv2.bias for block 1, then holomorphic, nblocks,
    channels, kernel_size -- the records equinox writes for the reference's model."""
    model = square4.model.ResConv(2, 8, seed=1)
    p = np.arange(model.nparams, dtype=np.float32) / 1000
    buf = io.BytesIO()
    ck.save_model(buf, model, p)
    recs = _records(buf)
    shapes = [r.shape for r in recs]
    assert shapes == [(8, 1, 3, 3), (8, 1, 1), (8, 8, 3, 3), (8, 1, 1), (8, 8, 3, 3), (8, 1, 1), (8, 8, 3, 3),
                      (), (), (), ()]
    assert all(r.dtype == np.float32 for r in recs[:7])
    assert recs[7].dtype == np.bool_ and not recs[7].item()
    assert [r.item() for r in recs[8:]] == [2, 8, 3]
    np.testing.assert_array_equal(np.concatenate([r.reshape(-1) for r in recs[:7]]), p)
    buf.seek(0)
    np.testing.assert_array_equal(ck.load_model(buf, model), p)


def test_reference_written_resconv_loads(square4):
    """A file holding the reference model's leaves (written here record by record, float64
    parameters as a float64 default dtype would give) loads as the flat parameter vector."""
    model = square4.model.ResConv(2, 4, seed=2)
    rng = np.random.default_rng(0)
    leaves = [rng.normal(size=(4, 1, 3, 3)), rng.normal(size=(4, 1, 1)), rng.normal(size=(4, 4, 3, 3)),
              rng.normal(size=(4, 1, 1)), rng.normal(size=(4, 4, 3, 3)), rng.normal(size=(4, 1, 1)),
              rng.normal(size=(4, 4, 3, 3))]
    buf = io.BytesIO()
    for x in leaves + [False, 2, 4, 3]:
        np.save(buf, x)
    buf.seek(0)
    got = ck.load_model(buf, model)
    np.testing.assert_array_equal(got, np.concatenate([x.reshape(-1) for x in leaves]).astype(np.float32))


def test_mismatched_checkpoint_is_refused(square4):
    model = square4.model.ResConv(2, 4, seed=2)
    other = square4.model.ResConv(2, 8, seed=2)
    buf = io.BytesIO()
    ck.save_model(buf, other, other.init_params)
    buf.seek(0)
    with pytest.raises(ValueError, match="shape"):
        ck.load_model(buf, model)
    # same shapes, different scalar leaf
    buf = io.BytesIO()
    for x in [np.zeros(s, np.float32) for _, s in ck.model_layout(model)[0]] + [False, 3, 4, 3]:
        np.save(buf, x)
    buf.seek(0)
    with pytest.raises(ValueError, match="nblocks"):
        ck.load_model(buf, model)
    buf = io.BytesIO()
    np.save(buf, np.zeros((4, 1, 3, 3), np.float32))
    buf.seek(0)
    with pytest.raises(ValueError, match="ends at record"):
        ck.load_model(buf, model)


def test_rbm_layout_and_flat_form():
    import quantax_gb300 as qtx
    qtx.set_default_dtype(np.float64)
    qtx.sites.Chain(8)
    model = qtx.model.RBM_Dense(3, init_std=0.1, seed=4)
    arrays, numbers = ck.model_layout(model)
    assert arrays == [("layers[0].weight", (3, 8)), ("layers[0].bias", (3,))] and numbers == [("holomorphic", False)]
    buf = io.BytesIO()
    ck.save_model(buf, model, model.init_params)
    recs = _records(buf)
    assert [r.shape for r in recs] == [(3, 8), (3,), ()]
    np.testing.assert_array_equal(recs[0].reshape(-1), model.init_params[:24])
    # the flat form (one array of every parameter) still loads
    flat = io.BytesIO()
    np.save(flat, model.init_params)
    flat.seek(0)
    np.testing.assert_array_equal(ck.load_model(flat, model), model.init_params)
    # no bias: the reference writes the weight only; the bias entries load as zeros
    nb = qtx.model.RBM_Dense(3, use_bias=False, init_std=0.1, seed=4)
    buf = io.BytesIO()
    ck.save_model(buf, nb, nb.init_params)
    assert [r.shape for r in _records(buf)] == [(3, 8), ()]
    buf.seek(0)
    got = ck.load_model(buf, nb)
    assert got.size == nb.nparams and not got[24:].any()


def test_optimizer_leaf_records():
    """The momentum optimizers' files: (mu, last_step) for SPRING, (mu, beta, m, v, t) for
    AdamSR, numbers as 0-d records (sr.py:258-262, 424-429)."""
    buf = io.BytesIO()
    ck.write_leaves(buf, [0.95, 0.995, np.arange(5.0), np.ones(5), 7])
    buf.seek(0)
    mu, beta, m, v, t = ck.read_leaves(buf, 5)
    assert (mu.item(), beta.item(), t.item()) == (0.95, 0.995, 7)
    assert mu.dtype == np.float64 and t.dtype.kind == "i"
    np.testing.assert_array_equal(m, np.arange(5.0))


def test_rbm_conv_record_sequence():
    """RBM_Conv on a 10 x 10 lattice: Conv.weight (C, 1, 10, 10), Conv.bias (C, 1, 1), holomorphic;
    on a chain Conv.bias is (C, 1)."""
    import quantax_gb300 as qtx
    qtx.set_default_dtype(np.float64)
    qtx.sites.Square(10)
    model = qtx.model.RBM_Conv(16, seed=1)
    buf = io.BytesIO()
    ck.save_model(buf, model, model.init_params)
    assert [r.shape for r in _records(buf)] == [(16, 1, 10, 10), (16, 1, 1), ()]
    buf.seek(0)
    np.testing.assert_array_equal(ck.load_model(buf, model), model.init_params)
    qtx.sites.Chain(12)
    chain = qtx.model.RBM_Conv(2, seed=1)
    buf = io.BytesIO()
    ck.save_model(buf, chain, chain.init_params)
    assert [r.shape for r in _records(buf)] == [(2, 1, 12), (2, 1), ()]
