"""ResConv in FP64 on the CPU (test infrastructure only).

Restates quantax/model/conv_nets.py:26-183 with nn/conv.py:13-68 and nn/activation.py:26-72:
  input (1, L, L) = spins as float (ReshapeConv)
  block b: residual = x; h = x / sqrt(b + 1); block 0: h /= sqrt(2), else h = gelu(h);
           h = conv1(h); h = gelu(h); h = conv2(h) (no bias in the last block's conv2);
           x = h + residual (block 0: residual repeated over the channels)
  final:   x /= sqrt(nblocks + 1); complex output: z = x[:C/2] + i x[C/2:] (pair_cpl);
           psi = mean_{c, r} exp(z)  (exp_by_scale + ConvSymmetrize with TransND, sector 0)
  convolutions: 3x3, SAME, circular padding, cross-correlation (equinox Conv);
  gelu: tanh approximation (jax.nn.gelu default).
log psi = logsumexp(z) - log(C' N); O = d log psi / d params (complex for complex output),
the vjp of quantax/state/variational.py:424-495, computed with torch autograd.
Parameter order: per block conv1.weight (C, Cin, 3, 3), conv1.bias (C, 1, 1), conv2.weight,
conv2.bias (absent in the last block) -- the ravel_pytree order of the equinox model.
"""
from __future__ import annotations

import math

import numpy as np
import torch
import torch.nn.functional as F


def shapes(nblocks, channels, kernel=3):
    out = []
    for b in range(nblocks):
        cin = 1 if b == 0 else channels
        out.append((channels, cin, kernel, kernel))
        out.append((channels, 1, 1))
        out.append((channels, channels, kernel, kernel))
        if b != nblocks - 1:
            out.append((channels, 1, 1))
    return out


def nparams(nblocks, channels, kernel=3):
    return int(sum(np.prod(s) for s in shapes(nblocks, channels, kernel)))


def init_he(nblocks, channels, seed=0, kernel=3, bias_std=0.0):
    """He-normal weights (fan_in = Cin * k * k); zero biases unless bias_std > 0."""
    rng = np.random.default_rng(seed)
    flat = []
    for s in shapes(nblocks, channels, kernel):
        if len(s) == 4:
            fan_in = s[1] * s[2] * s[3]
            flat.append(rng.normal(0.0, math.sqrt(2.0 / fan_in), s).ravel())
        else:
            flat.append(rng.normal(0.0, bias_std, s).ravel() if bias_std > 0 else np.zeros(int(np.prod(s))))
    return np.concatenate(flat).astype(np.float32)


def gelu(x):
    return 0.5 * x * (1.0 + torch.tanh(math.sqrt(2.0 / math.pi) * (x + 0.044715 * x ** 3)))


def _unflatten(p, nblocks, channels, kernel=3):
    out, off = [], 0
    for s in shapes(nblocks, channels, kernel):
        n = int(np.prod(s))
        out.append(p[off:off + n].reshape(s))
        off += n
    return out


def _conv(x, w, b):
    xp = F.pad(x, (1, 1, 1, 1), mode="circular")
    y = F.conv2d(xp, w)
    return y if b is None else y + b.reshape(1, -1, 1, 1)


def features(p, spins, L, nblocks, channels):
    """x after the last block and the final 1/sqrt(nblocks + 1) scaling: (ns, C, L, L)."""
    ws = _unflatten(p, nblocks, channels)
    x = spins.reshape(-1, 1, L, L)
    k = 0
    for b in range(nblocks):
        res = x
        h = x / math.sqrt(b + 1)
        h = h / math.sqrt(2.0) if b == 0 else gelu(h)
        w1, b1 = ws[k], ws[k + 1]
        k += 2
        h = gelu(_conv(h, w1, b1))
        w2 = ws[k]
        b2 = ws[k + 1] if b != nblocks - 1 else None
        k += 2 if b != nblocks - 1 else 1
        h = _conv(h, w2, b2)
        if res.shape[1] < h.shape[1]:
            res = res.repeat(1, h.shape[1] // res.shape[1], 1, 1)
        x = h + res
    return x / math.sqrt(nblocks + 1)


def log_psi_torch(p, spins, L, nblocks, channels, complex_out=True, sinhp1=False):
    """log of the mean final activation: exp_by_scale, or sinhp1_by_scale (sinh z + 1) when
    sinhp1 (quantax/nn/activation.py:7-32); complex for sinhp1 (a real psi can be negative)."""
    x = features(p, spins, L, nblocks, channels)
    ns = x.shape[0]
    if complex_out:
        c2 = channels // 2
        z = torch.complex(x[:, :c2], x[:, c2:]).reshape(ns, -1)
    else:
        z = x.reshape(ns, -1)
    if sinhp1:
        z = z.to(torch.complex128)
        m = z.real.abs().max(dim=1, keepdim=True).values
        sig = 0.5 * (torch.exp(z - m) - torch.exp(-z - m)) + torch.exp(-m)
        return m.squeeze(1) + torch.log(sig.sum(dim=1)) - math.log(z.shape[1])
    m = z.real.max(dim=1, keepdim=True).values
    lse = m.squeeze(1) + torch.log(torch.exp(z - m).sum(dim=1))
    return lse - math.log(z.shape[1])


class ResConv:
    def __init__(self, params, L, nblocks, channels, complex_out=True, sinhp1=False):
        self.p = np.asarray(params, dtype=np.float64)
        self.L, self.nblocks, self.channels, self.complex_out = L, nblocks, channels, complex_out
        self.sinhp1 = sinhp1

    def log_psi(self, s):
        s = torch.as_tensor(np.atleast_2d(s), dtype=torch.float64)
        p = torch.as_tensor(self.p)
        with torch.no_grad():
            lp = log_psi_torch(p, s, self.L, self.nblocks, self.channels, self.complex_out, self.sinhp1)
        return lp.numpy()

    def jacobian(self, s):
        """O (ns, np): complex128 for complex output (d Re log psi + i d Im log psi)."""
        s = torch.as_tensor(np.atleast_2d(s), dtype=torch.float64)
        rows = []
        for a in range(s.shape[0]):
            p = torch.as_tensor(self.p).clone().requires_grad_(True)
            lp = log_psi_torch(p, s[a:a + 1], self.L, self.nblocks, self.channels, self.complex_out,
                               self.sinhp1)[0]
            if self.complex_out:
                gr, = torch.autograd.grad(lp.real, p, retain_graph=True)
                gi, = torch.autograd.grad(lp.imag, p)
                rows.append((gr + 1j * gi).numpy())
            else:
                # real output: d log |psi| (a sinhp1 psi carries its sign in the phase)
                g, = torch.autograd.grad(lp.real, p)
                rows.append(g.numpy())
        return np.stack(rows)
