"""Philox4x32-10 counter-based generator and the random streams of the VMC loop.

Test infrastructure only: this module is the CPU checker for the CUDA path and is
never called by the product code.

The reference draws its randomness from JAX's threefry streams
(quantax/global_defs.py:54-91, quantax/sampler/common_samplers.py:28-33, 58-82,
quantax/sampler/metropolis.py:300-304).  JAX is not available to reproduce those
streams, so the GPU path and this oracle share one counter-based generator instead:
Philox4x32-10 as published by Salmon, Moraes, Dror and Shaw, "Parallel random
numbers: as easy as 1, 2, 3" (SC'11).  Ten rounds of

    (hi0, lo0) = mulhilo(0xD2511F53, c0)
    (hi1, lo1) = mulhilo(0xCD9E8D57, c2)
    c = (hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0)
    k = (k0 + 0x9E3779B9, k1 + 0xBB67AE85)       (between rounds)

The stream layout (which counter words carry which index) is this project's own and is
mirrored bit for bit by quantax_gb300/csrc/qgx_common.cuh.
"""
from __future__ import annotations

import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint32(0x9E3779B9)
W1 = np.uint32(0xBB67AE85)
MASK32 = np.uint64(0xFFFFFFFF)

# purpose tags carried in counter word 3 (bits 24..31); must match qgx_common.cuh
TAG_PROPOSE = 1      # Metropolis proposal + accept draw
TAG_INIT = 2         # initial configurations
TAG_INIT_PERM = 3    # fixed-magnetisation initial configurations
TAG_EXACT = 4        # draws of the exact sampler


def philox4x32_10(ctr, key):
    """Vectorised Philox4x32-10.

    ctr: uint32 array [..., 4]; key: uint32 array [..., 2] (broadcast).
    Returns uint32 array [..., 4].
    """
    c = np.array(ctr, dtype=np.uint32)
    k = np.array(key, dtype=np.uint32)
    c0 = c[..., 0].astype(np.uint64)
    c1 = c[..., 1].astype(np.uint64)
    c2 = c[..., 2].astype(np.uint64)
    c3 = c[..., 3].astype(np.uint64)
    k0 = np.broadcast_to(k[..., 0], c[..., 0].shape).astype(np.uint64)
    k1 = np.broadcast_to(k[..., 1], c[..., 0].shape).astype(np.uint64)
    for r in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK32
        c0 = (hi1 ^ c1 ^ k0) & MASK32
        c1 = lo1
        c2 = (hi0 ^ c3 ^ k1) & MASK32
        c3 = lo0
        if r < 9:
            k0 = (k0 + np.uint64(W0)) & MASK32
            k1 = (k1 + np.uint64(W1)) & MASK32
    return np.stack([c0, c1, c2, c3], axis=-1).astype(np.uint32)


def seed_key(seed: int):
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    return np.array([seed & 0xFFFFFFFF, seed >> 32], dtype=np.uint32)


def stream_counter(chain, step, tag, substream=0):
    """Counter of draw `step` of chain `chain`.

    c0 = chain index, c1 = low 32 bits of the step, c2 = high 32 bits of the step,
    c3 = tag << 24 | substream (substream < 2**24).
    """
    chain = np.asarray(chain, dtype=np.uint64)
    step = np.asarray(step, dtype=np.uint64)
    chain, step = np.broadcast_arrays(chain, step)
    c = np.empty(chain.shape + (4,), dtype=np.uint32)
    c[..., 0] = (chain & MASK32).astype(np.uint32)
    c[..., 1] = (step & MASK32).astype(np.uint32)
    c[..., 2] = (step >> np.uint64(32)).astype(np.uint32)
    c[..., 3] = np.uint32((int(tag) << 24) | (int(substream) & 0xFFFFFF))
    return c


def draw(seed, chain, step, tag, substream=0):
    return philox4x32_10(stream_counter(chain, step, tag, substream), seed_key(seed))


def bounded(word, n):
    """Map a uniform 32-bit word to {0..n-1} by the multiply-shift (w * n) >> 32."""
    return ((np.asarray(word, dtype=np.uint64) * np.uint64(n)) >> np.uint64(32)).astype(np.int64)


def unit_float(word):
    """Uniform float in [0, 1) with 24 random bits: (w >> 8) * 2**-24 (exact in fp32)."""
    return (np.asarray(word, dtype=np.uint32) >> np.uint32(8)).astype(np.float64) * (2.0 ** -24)


def unit_double(x, y):
    """Uniform float64 in [0, 1) with 53 random bits: ((x >> 5) 2**26 + (y >> 6)) 2**-53."""
    x = np.asarray(x, dtype=np.uint32) >> np.uint32(5)
    y = np.asarray(y, dtype=np.uint32) >> np.uint32(6)
    return (x.astype(np.float64) * 67108864.0 + y.astype(np.float64)) * (2.0 ** -53)
