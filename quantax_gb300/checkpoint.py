"""Checkpoints in the reference's file format.

quantax saves a model with equinox.tree_serialise_leaves (quantax/state/variational.py:162-163,
581-587) and an optimizer's momentum state the same way (quantax/optimizer/sr.py:244-263,
316-349, 398-429). That format (equinox >= 0.11.4, a dependency absent here) is a plain
concatenation of .npy records: one record per leaf of the pytree, in leaf order, for every
array and every Python / numpy number (bool, int, float, complex); other leaves (functions,
dtypes, None, static fields) are not written. Reading walks the same leaf order.

The leaf order of the two models follows from their dataclass fields:

  RBM_Dense = SingleDense (quantax/model/shallow_nets.py:35-78): layers = (Linear, Lambda,
    prod_by_log), holomorphic  ->  Linear.weight (M, N), Linear.bias (M,) [use_bias], holomorphic.
  RBM_Conv = SingleConv (shallow_nets.py:129-170): layers = (ReshapeConv, Conv, Lambda,
    prod_by_log), holomorphic  ->  Conv.weight (C, 1, *lattice), Conv.bias (C, 1[, 1]), holomorphic.
  ResConv (quantax/model/conv_nets.py:95-183): fields layers, holomorphic (from Sequential,
    quantax/nn/modules.py:9-37), then nblocks, channels, kernel_size, final_activation,
    trans_symm, dtype, out_dtype; layers = (ReshapeConv, _ConvBlock..., final layer,
    ConvSymmetrize), each block conv1, conv2 (equinox Conv: weight (C, Cin, k, k), bias (C, 1, 1),
    absent in the last block's conv2)  ->  the conv records block by block, then holomorphic,
    nblocks, channels, kernel_size.

The flat parameter vector of quantax_gb300 is the concatenation of the array records
(jax.flatten_util.ravel_pytree order, quantax/state/variational.py:241), so loading is a
concatenation and saving a split.
"""
from __future__ import annotations

from typing import BinaryIO, List, Sequence, Tuple, Union

import numpy as np

PathOrFile = Union[str, "os.PathLike", BinaryIO]


def model_layout(model) -> Tuple[List[Tuple[str, tuple]], List[Tuple[str, object]]]:
    """(array leaves as (name, shape), number leaves as (name, value)) of a model."""
    kind = getattr(model, "kind", None)
    if kind == "rbm" and getattr(model, "conv", False):
        # SingleConv: layers = (ReshapeConv, Conv, Lambda, prod_by_log), holomorphic
        dims = (model.L0,) if model.L1 == 1 else (model.L0, model.L1)
        arrays = [("layers[1].weight", (model.channels, 1) + dims)]
        if model.use_bias:
            arrays.append(("layers[1].bias", (model.channels,) + (1,) * len(dims)))
        return arrays, [("holomorphic", False)]
    if kind == "rbm":
        if getattr(model, "visible_bias", False):
            raise ValueError("the reference's RBM_Dense has no visible bias: no checkpoint layout")
        arrays = [("layers[0].weight", (model.M, model.N))]
        if model.use_bias:
            arrays.append(("layers[0].bias", (model.M,)))
        return arrays, [("holomorphic", False)]
    if kind == "resconv":
        C = model.channels
        arrays = []
        for b in range(model.nblocks):
            cin = 1 if b == 0 else C
            arrays.append((f"layers[{b + 1}].conv1.weight", (C, cin, 3, 3)))
            arrays.append((f"layers[{b + 1}].conv1.bias", (C, 1, 1)))
            arrays.append((f"layers[{b + 1}].conv2.weight", (C, C, 3, 3)))
            if b != model.nblocks - 1:
                arrays.append((f"layers[{b + 1}].conv2.bias", (C, 1, 1)))
        return arrays, [("holomorphic", False), ("nblocks", model.nblocks), ("channels", C), ("kernel_size", 3)]
    raise ValueError(f"no checkpoint layout for {type(model).__name__}")


def _open(file, mode):
    if hasattr(file, "read") or hasattr(file, "write"):
        return file, False
    return open(file, mode), True


def write_leaves(file: PathOrFile, leaves: Sequence) -> None:
    """np.save every array / number leaf in order (equinox's serialise filter)."""
    f, own = _open(file, "wb")
    try:
        for x in leaves:
            np.save(f, x, allow_pickle=False)
    finally:
        if own:
            f.close()


def read_leaves(file: PathOrFile, count: int) -> list:
    """The first `count` .npy records of the file."""
    f, own = _open(file, "rb")
    try:
        out = []
        for i in range(count):
            try:
                out.append(np.load(f, allow_pickle=False))
            except (EOFError, ValueError) as e:
                raise ValueError(f"checkpoint ends at record {i}, {count} expected") from e
        return out
    finally:
        if own:
            f.close()


def save_model(file: PathOrFile, model, params: np.ndarray) -> None:
    """The model's parameters (flat, float32) in the reference's layout."""
    arrays, numbers = model_layout(model)
    p = np.asarray(params, dtype=np.float32).reshape(-1)
    leaves, off = [], 0
    for name, shape in arrays:
        n = int(np.prod(shape))
        leaves.append(p[off:off + n].reshape(shape))
        off += n
    if model.kind == "rbm" and not model.use_bias:
        # the bias entries kept at zero here are not leaves of the reference model
        off += model.channels if getattr(model, "conv", False) else model.M
    if off != p.size:
        raise ValueError(f"{p.size} parameters, the layout holds {off}")
    leaves += [v for _, v in numbers]
    write_leaves(file, leaves)


def load_model(file: PathOrFile, model) -> np.ndarray:
    """Flat float32 parameters from a file in the reference's layout, or from a single .npy
    array of all parameters (the flat form)."""
    arrays, numbers = model_layout(model)
    f, own = _open(file, "rb")
    try:
        first = np.load(f, allow_pickle=False)
        if first.ndim == 1 and first.size == model.nparams:
            return first.astype(np.float32)  # flat form
        recs = [first] + read_leaves(f, len(arrays) + len(numbers) - 1)
    finally:
        if own:
            f.close()
    parts = []
    for (name, shape), r in zip(arrays, recs):
        if tuple(r.shape) != tuple(shape):
            raise ValueError(f"{name}: shape {tuple(r.shape)} in the file, the model has {tuple(shape)}")
        if np.iscomplexobj(r):
            raise ValueError(f"{name}: complex parameters are not supported")
        parts.append(np.asarray(r, dtype=np.float32).reshape(-1))
    if model.kind == "rbm" and not model.use_bias:
        parts.append(np.zeros(model.channels if getattr(model, "conv", False) else model.M, dtype=np.float32))
    for (name, want), r in zip(numbers, recs[len(arrays):]):
        got = r.item()
        if got != want:
            raise ValueError(f"{name} = {got!r} in the file, the model has {want!r}")
    return np.concatenate(parts)
