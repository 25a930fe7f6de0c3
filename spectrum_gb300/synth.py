"""Seeded synthetic beams with the shapes and value distributions of the
benchmark workloads (the reference publishes no dataset; all inputs are
synthetic).

Each beam is a sum of complex tones plus circular complex Gaussian noise:

    x[n] = sum_t A_t exp(i (2 pi f_t n + phi_t)) + sigma (g1 + i g2) / sqrt(2)

with f_t ~ U[0, 0.5) cycles/sample, A_t log-uniform in [0.1, 1],
phi_t ~ U[0, 2 pi).  Where a workload gives an SNR, sigma = max_t A_t *
10^(-SNR/20) (SNR of the strongest tone against the total noise power).
Tone parameters come from numpy's PCG64 seeded per workload; the samples are
synthesised in FP64 and stored as complex64, on the CPU (numpy) or on a CUDA
device (torch, noise from a seeded torch.Generator).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class BeamSet:
    lengths: np.ndarray        # [beams] samples per beam
    freqs: list                # per beam: array of tone frequencies (cycles/sample)
    amps: list                 # per beam: tone amplitudes
    phases: list               # per beam: tone phases (rad)
    sigma: np.ndarray          # [beams] noise std (complex)
    seed: int

    @property
    def beams(self) -> int:
        return len(self.lengths)


def _tones(rng, n):
    f = rng.uniform(0.0, 0.5, n)
    a = np.exp(rng.uniform(np.log(0.1), np.log(1.0), n))
    p = rng.uniform(0.0, 2 * np.pi, n)
    return f, a, p


def make_beams(lengths, tones=(1, 1), sigma=None, snr_db=None, seed=0) -> BeamSet:
    """tones=(lo, hi): tone count per beam uniform in [lo, hi]; give either a
    fixed noise sigma or an SNR range (lo_db, hi_db)."""
    rng = np.random.default_rng(seed)
    lengths = np.asarray(lengths, dtype=np.int64)
    fs, as_, ps, sig = [], [], [], np.zeros(len(lengths))
    for b in range(len(lengths)):
        n = int(rng.integers(tones[0], tones[1] + 1))
        f, a, p = _tones(rng, n)
        fs.append(f)
        as_.append(a)
        ps.append(p)
        if snr_db is not None:
            snr = rng.uniform(snr_db[0], snr_db[1])
            sig[b] = a.max() * 10.0 ** (-snr / 20.0)
        else:
            sig[b] = float(sigma or 0.0)
    return BeamSet(lengths, fs, as_, ps, sig, seed)


# ---- the benchmark workloads -------------------------------------------------
def workload_small(seed: int = 0) -> BeamSet:
    """8 beams x 4096, 3 tones, sigma 0.01 (nFFT 4096, Hann, top-5)."""
    return make_beams([4096] * 8, tones=(3, 3), sigma=0.01, seed=seed)


def workload_large(seed: int = 1, beams: int = 256) -> BeamSet:
    """256 beams x 65536, 1-16 tones, SNR U[0, 40] dB (nFFT 131072, all maxima > 6 sigma)."""
    return make_beams([65536] * beams, tones=(1, 16), snr_db=(0.0, 40.0), seed=seed)


def workload_uneven(seed: int = 2, beams: int = 1024) -> BeamSet:
    """1024 beams, lengths U[1000, 100000], 1-8 tones, SNR U[0, 40] dB (top-8)."""
    rng = np.random.default_rng(seed + 1000)
    lengths = rng.integers(1000, 100001, beams)
    return make_beams(lengths, tones=(1, 8), snr_db=(0.0, 40.0), seed=seed)


def workload_precision(seed: int = 3, beams: int = 64, n: int = 1 << 20):
    """64 beams x 2^20: two tones 120 dB apart + noise sigma 1e-7 (Blackman-Harris)."""
    rng = np.random.default_rng(seed)
    fs, as_, ps = [], [], []
    for _ in range(beams):
        f = rng.uniform(0.0, 0.5, 2)
        a = np.array([1.0, 1e-6])
        p = rng.uniform(0.0, 2 * np.pi, 2)
        fs.append(f)
        as_.append(a)
        ps.append(p)
    return BeamSet(np.full(beams, n, np.int64), fs, as_, ps, np.full(beams, 1e-7), seed)


def workload_learned(seed: int = 4, beams: int = 4096, n: int = 8192, snr_db: float = 20.0) -> BeamSet:
    """4096 beams x 8192, one tone each at a fixed SNR (learned-refinement inference)."""
    return make_beams([n] * beams, tones=(1, 1), snr_db=(snr_db, snr_db), seed=seed)


# ---- synthesis -----------------------------------------------------------------
def synth_numpy(bs: BeamSet, pad_to: int | None = None) -> np.ndarray:
    """Rows of length max(lengths) (or pad_to), zero beyond each beam's length."""
    width = int(pad_to or bs.lengths.max())
    out = np.zeros((bs.beams, width), np.complex64)
    rng = np.random.default_rng(bs.seed + 7919)
    for b in range(bs.beams):
        n = int(bs.lengths[b])
        t = np.arange(n, dtype=np.float64)
        x = np.zeros(n, np.complex128)
        for f, a, p in zip(bs.freqs[b], bs.amps[b], bs.phases[b]):
            x += a * np.exp(1j * (2 * np.pi * np.mod(f * t, 1.0) + p))
        if bs.sigma[b] > 0:
            x += bs.sigma[b] * (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2)
        out[b, :n] = x.astype(np.complex64)
    return out


def synth_torch(bs: BeamSet, device="cuda", packed: bool = True):
    """On-device synthesis.  packed=True returns one flat complex64 tensor with
    the beams back to back (the layout of uneven batches); for equal lengths
    it is reshaped to [beams, n]."""
    import torch

    gen = torch.Generator(device=device)
    gen.manual_seed(int(bs.seed) + 7919)
    parts = []
    for b in range(bs.beams):
        n = int(bs.lengths[b])
        t = torch.arange(n, dtype=torch.float64, device=device)
        f = torch.as_tensor(bs.freqs[b], dtype=torch.float64, device=device)
        a = torch.as_tensor(bs.amps[b], dtype=torch.float64, device=device)
        p = torch.as_tensor(bs.phases[b], dtype=torch.float64, device=device)
        ph = 2 * np.pi * torch.remainder(f[:, None] * t[None, :], 1.0) + p[:, None]
        re = (a[:, None] * torch.cos(ph)).sum(0)
        im = (a[:, None] * torch.sin(ph)).sum(0)
        if bs.sigma[b] > 0:
            s = float(bs.sigma[b]) / np.sqrt(2)
            re = re + s * torch.randn(n, generator=gen, dtype=torch.float64, device=device)
            im = im + s * torch.randn(n, generator=gen, dtype=torch.float64, device=device)
        parts.append(torch.complex(re.float(), im.float()))
    flat = torch.cat(parts)
    if packed and len(set(int(v) for v in bs.lengths)) == 1:
        return flat.reshape(bs.beams, int(bs.lengths[0]))
    return flat
