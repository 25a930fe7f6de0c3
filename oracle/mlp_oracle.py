"""CPU oracle for the learned sub-bin refinement (FP64 numpy).

TEST INFRASTRUCTURE ONLY.  Only ``tests/`` and the CPU legs of ``bench.py``
may import this module, as the checker; the product path never calls it.

The learned refinement has no reference counterpart: it stands beside the
3-point parabola of post_kernel_one_peak
(include/spectrum/kernels/fft_kernel_sources_rocm.hpp:228-239).  This module
defines the network the CUDA kernels implement and serves as the gradient
check for them:

* 10 -> 64 -> 64 -> 2, GELU(z) = z/2 (1 + erf(z/sqrt 2)) after both hidden
  layers; parameters W1[64][10] b1 W2[64][64] b2 W3[2][64] b3 (4994 floats);
  the products use the BF16 rounding (nearest, ties to even) of the weights;
* loss = sum over the rows with mask != 0 of |y - t|^2, divided by rows * 2
  (masked-out rows count in the denominator and add 0);
* Adam with beta1 0.9, beta2 0.999, eps 1e-8 and bias correction;
* features of the peak at bin k: |X[k+d]|/|X[k]| and
  wrap(arg(X[k+d] conj X[k]) + pi d (n_point - 1)/nfft), d = -2..2;
* labels: the fine-grid peak of a 16x zero-padded FFT within +-24 fine bins
  of 16k, refined by a 3-point parabola on the fine grid.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

N_IN, N_H, N_OUT = 10, 64, 2
SHAPES = [(N_H, N_IN), (N_H,), (N_H, N_H), (N_H,), (N_OUT, N_H), (N_OUT,)]
N_PARAMS = sum(int(np.prod(s)) for s in SHAPES)


def bf16_round(x) -> np.ndarray:
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def unpack(p, round_weights: bool = True):
    """Parameter vector -> [W1, b1, W2, b2, W3, b3] as float64 (weights BF16-rounded)."""
    p = np.asarray(p, np.float32 if round_weights else np.float64)
    out, off = [], 0
    for i, s in enumerate(SHAPES):
        n = int(np.prod(s))
        v = p[off:off + n]
        if i % 2 == 0 and round_weights:
            v = bf16_round(v)
        out.append(v.astype(np.float64).reshape(s))
        off += n
    return out


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def forward(p, x, round_weights: bool = True):
    W1, b1, W2, b2, W3, b3 = unpack(p, round_weights)
    x = np.asarray(x, np.float64)
    z1 = x @ W1.T + b1
    h1 = gelu(z1)
    z2 = h1 @ W2.T + b2
    h2 = gelu(z2)
    y = h2 @ W3.T + b3
    return y, (x, z1, h1, z2, h2)


def loss_and_grad(p, x, t, mask=None, round_weights: bool = True):
    """-> (loss, gradient vector in parameter order), FP64."""
    W1, b1, W2, b2, W3, b3 = unpack(p, round_weights)
    y, (x, z1, h1, z2, h2) = forward(p, x, round_weights)
    rows = y.shape[0]
    m = np.ones(rows) if mask is None else (np.asarray(mask) != 0).astype(np.float64)
    d = (y - np.asarray(t, np.float64)) * m[:, None]
    loss = float((d * d).sum() / (rows * N_OUT))
    dy = d * (2.0 / (rows * N_OUT))
    gW3 = dy.T @ h2
    gb3 = dy.sum(0)
    dz2 = (dy @ W3) * gelu_grad(z2)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * gelu_grad(z1)
    gW1 = dz1.T @ x
    gb1 = dz1.sum(0)
    return loss, np.concatenate([g.ravel() for g in (gW1, gb1, gW2, gb2, gW3, gb3)])


def adam_step(p, m, v, g, lr, step, b1=0.9, b2=0.999, eps=1e-8):
    """One bias-corrected Adam step (FP64) -> (p, m, v)."""
    p, m, v, g = (np.asarray(a, np.float64) for a in (p, m, v, g))
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v


def peak_features(spec, k, n_point, nfft):
    """Features of the peak at bin k of one spectrum (complex array), FP64."""
    spec = np.asarray(spec, np.complex128)
    c = spec[k]
    d = np.arange(-2, 3)
    z = spec[k + d]
    mag = np.abs(z) / np.abs(c)
    ph = np.angle(z * np.conj(c)) + np.pi * d * (n_point - 1) / nfft
    ph = ph - 2 * np.pi * np.rint(ph / (2 * np.pi))
    ph[2] = 0.0
    return np.concatenate([mag, ph])


def fine_label(spec16, k, spec):
    """(offset in bins, log(amplitude/|X[k]|)) from the 16x zero-padded spectrum."""
    g = np.abs(np.asarray(spec16, np.complex128))
    m = 16 * k + np.arange(-24, 25)
    mb = int(m[np.argmax(g[m])])
    yl, yc, yr = g[mb - 1], g[mb], g[mb + 1]
    den = yl - 2 * yc + yr
    df = float(np.clip(0.5 * (yl - yr) / den, -0.5, 0.5)) if abs(den) > 1e-20 else 0.0
    amp = yc - 0.25 * (yl - yr) * df
    return (mb - 16 * k + df) / 16.0, float(np.log(amp / abs(spec[k])))


def hann(n_point):
    t = np.arange(n_point)
    return 0.5 * (1.0 - np.cos(2.0 * np.pi * t / (n_point - 1)))
