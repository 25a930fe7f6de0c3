"""Generates the golden fixtures of tests/golden/ from the reference itself.

Runs only where oracle/_ref exists (built by oracle/build_ref.py from the
reference sources): the reference's CpuFFT (pocketfft) and its peak-search /
magnitude kernel text executed on the CPU.  Inputs are seeded; the outputs
are the reference's, byte for byte.  Re-run with

    python tests/golden/make_golden.py

The fixtures are small (< 1 MB) and read by tests/test_oracle_golden.py.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle import reference_lib as ref  # noqa: E402


def _spec(rng, beams, n, ties):
    if ties:
        return (rng.integers(-3, 4, (beams, n)) + 1j * rng.integers(-3, 4, (beams, n))).astype(np.complex64)
    z = (rng.standard_normal((beams, n)) + 1j * rng.standard_normal((beams, n))).astype(np.complex64)
    for b in range(beams):  # a few strong lines
        for k in rng.integers(2, n - 2, 3):
            z[b, k] += np.complex64(50 * np.exp(1j * rng.uniform(0, 6.28)))
    return z


def main():
    assert ref.available(), "oracle/_ref missing: run oracle/build_ref.py (needs the reference sources)"
    rng = np.random.default_rng(20261203)
    out = {}

    # 1. ONE_PEAK / TWO_PEAKS (post kernels), incl. exact ties
    cases = [(1024, 0, False), (1024, 1024, True), (2048, 300, False), (2048, 0, True), (4096, 2, False)]
    for i, (nfft, sr, ties) in enumerate(cases):
        z = _spec(rng, 2, nfft, ties)
        for two in (0, 1):
            key = f"post{i}_{two}"
            out[f"{key}_fft"] = z
            out[f"{key}_meta"] = np.array([nfft, sr, two, 10000], np.int64)
            out[f"{key}_out"] = ref.post_peaks(z, nfft, sr, 10000.0, bool(two)).view(np.uint32)

    # 2. ALL_MAXIMA pipeline (detect -> Blelloch scan -> compact)
    cases = [(1024, 0, 0, 1000, False), (4096, 5, 4096, 50, True), (4096, 0, 0, 100000, False),
             (2048, 3000, 100, 1000, False), (2048, 1, 3, 1000, True), (1536, 0, 0, 1000, True)]
    for i, (nfft, s, e, cap, ties) in enumerate(cases):
        z = _spec(rng, 2, nfft, ties)
        m = ref.compute_magnitudes(z)
        res, counts = ref.all_maxima(m, z, nfft, 48000.0, s, e, cap)
        key = f"all{i}"
        out[f"{key}_fft"] = z
        out[f"{key}_mag"] = m
        out[f"{key}_meta"] = np.array([nfft, s, e, cap, 48000], np.int64)
        out[f"{key}_counts"] = counts
        rows = [res[b, : min(int(counts[b]), res.shape[1])] for b in range(2)]
        out[f"{key}_out0"] = rows[0].view(np.uint32)
        out[f"{key}_out1"] = rows[1].view(np.uint32)

    # 3. magnitude / mag-phase kernels
    z = _spec(rng, 1, 999, False)[0]
    out["mag_z"] = z
    out["mag_out"] = ref.complex_to_magnitude(z, 1.0 / 999, False)
    out["mag2_out"] = ref.complex_to_magnitude(z, 0.5, True)
    out["magphase_out"] = ref.complex_to_mag_phase(z)

    # 4. CpuFFT::ForwardC2C
    for n in (64, 1000, 4096, 4374):
        x = _spec(rng, 2, n, False)
        out[f"fft{n}_x"] = x
        out[f"fft{n}_X"] = ref.cpu_fft_c2c(x)

    # 5. known answer: 100 Hz sine, fs 10 kHz, 1000 points, nFFT 1024 (ONE_PEAK)
    t = np.arange(1000)
    x = np.exp(2j * np.pi * 100.0 * t / 10000.0).astype(np.complex64)
    X = np.zeros(1024, np.complex64)
    X[:] = ref.cpu_fft_c2c(np.concatenate([x, np.zeros(24, np.complex64)])[None])[0]
    out["kat100_X"] = X
    out["kat100_out"] = ref.post_peaks(X[None], 1024, 0, 10000.0, False).view(np.uint32)

    # 6. CpuFFT::InverseC2C, ForwardR2C, ForwardR2C_Full
    for n in (64, 1000, 4096):
        x = _spec(rng, 2, n, False)
        out[f"ifft{n}_X"] = x
        out[f"ifft{n}_x"] = ref.cpu_ifft_c2c(x)
        r = rng.standard_normal((2, n)).astype(np.float32)
        out[f"r2c{n}_x"] = r
        out[f"r2c{n}_half"] = ref.cpu_fft_r2c(r, False)
        out[f"r2c{n}_full"] = ref.cpu_fft_r2c(r, True)

    np.savez_compressed(HERE / "reference_golden.npz", **out)
    print(f"wrote {HERE / 'reference_golden.npz'} ({(HERE / 'reference_golden.npz').stat().st_size} bytes)")


if __name__ == "__main__":
    main()
