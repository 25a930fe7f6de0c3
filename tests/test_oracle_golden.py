"""Pins the oracle (oracle/spectrum_oracle.py) to the reference.

1. Against tests/golden/reference_golden.npz, produced by the reference's own
   kernel text and CpuFFT run here (tests/golden/make_golden.py): peak lists
   bit-exact (phase within 1e-4 degree: host atan2f vs the oracle's numpy),
   magnitudes bit-exact, FFT within 1e-6 of the spectrum peak (two pocketfft
   builds differ in the last bits).
2. Against the reference's known-answer tests (tests/test_spectrum_maxima_rocm.hpp,
   tests/test_complex_to_mag_phase_rocm.hpp).
3. Against the live reference (oracle/_ref) on fresh random cases, where it
   was built.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import spectrum_oracle as orc

G = np.load(Path(__file__).parent / "golden" / "reference_golden.npz")
EXACT = ["index", "real", "imag", "magnitude", "freq_offset", "refined_frequency", "pad"]


def _mv(words):
    return np.ascontiguousarray(words).view(orc.MAXVALUE_DTYPE)


def assert_mv_equal(a, b):
    for f in EXACT:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)
    np.testing.assert_allclose(a["phase"], b["phase"], atol=1e-4, rtol=0)


@pytest.mark.parametrize("i", range(5))
@pytest.mark.parametrize("two", [0, 1])
def test_post_peaks_golden(i, two):
    key = f"post{i}_{two}"
    nfft, sr, _, fs = G[f"{key}_meta"]
    ref = _mv(G[f"{key}_out"]).reshape(-1)
    got = orc.one_two_peaks(G[f"{key}_fft"], int(nfft), int(sr), float(fs), bool(two)).reshape(-1)
    assert_mv_equal(got, ref)


@pytest.mark.parametrize("i", range(6))
def test_all_maxima_golden(i):
    key = f"all{i}"
    nfft, s, e, cap, fs = (int(v) for v in G[f"{key}_meta"])
    mag, fft = G[f"{key}_mag"], G[f"{key}_fft"]
    np.testing.assert_array_equal(orc.mag_rn(fft), mag)
    got, counts = orc.all_maxima(mag, fft, nfft, float(fs), s, e, cap)
    np.testing.assert_array_equal(counts, G[f"{key}_counts"])
    for b in range(2):
        ref = _mv(G[f"{key}_out{b}"]).reshape(-1)
        assert_mv_equal(got[b, : len(ref)], ref)


def test_magnitude_golden():
    z = G["mag_z"]
    np.testing.assert_array_equal(orc.magnitude(z, np.float32(1.0 / 999)), G["mag_out"])
    np.testing.assert_array_equal(orc.magnitude(z, 0.5, squared=True), G["mag2_out"])
    mp = orc.mag_phase(z)
    np.testing.assert_array_equal(mp[:, 0], G["magphase_out"][:, 0])
    np.testing.assert_allclose(mp[:, 1], G["magphase_out"][:, 1], atol=1e-6, rtol=0)


@pytest.mark.parametrize("n", [64, 1000, 4096, 4374])
def test_fft_matches_reference_cpufft(n):
    x, X = G[f"fft{n}_x"], G[f"fft{n}_X"]
    got = orc.fft_fp32(x, n)
    err = np.abs(got - X).max() / np.abs(X).max()
    assert err < 1e-6, err


@pytest.mark.parametrize("n", [64, 1000, 4096])
def test_inverse_and_real_ffts_match_reference_cpufft(n):
    """CpuFFT::InverseC2C / ForwardR2C / ForwardR2C_Full of the reference
    (golden) against the oracle's restatement."""
    X, x = G[f"ifft{n}_X"], G[f"ifft{n}_x"]
    assert np.abs(orc.ifft_fp32(X) - x).max() / np.abs(x).max() < 1e-6
    r, half, full = G[f"r2c{n}_x"], G[f"r2c{n}_half"], G[f"r2c{n}_full"]
    assert half.shape == (2, n // 2 + 1) and full.shape == (2, n)
    assert np.abs(orc.fft_r2c_fp32(r, n) - half).max() / np.abs(half).max() < 1e-6
    got_full = orc.fft_r2c_fp32(r, n, full=True)
    assert np.abs(got_full - full).max() / np.abs(full).max() < 1e-6
    k = np.arange(n // 2 + 1, n)   # the reference's mirror is exact
    np.testing.assert_array_equal(full[:, k], np.conj(full[:, n - k]))


def test_known_answer_100hz():
    """tests/test_spectrum_maxima_rocm.hpp:98-126: 100 Hz, fs 10 kHz, 1000 pts -> |f - 100| < 5 Hz."""
    ref = _mv(G["kat100_out"]).reshape(-1)
    got = orc.one_two_peaks(G["kat100_X"][None], 1024, 0, 10000.0, False).reshape(-1)
    assert_mv_equal(got, ref)
    assert abs(got[0]["refined_frequency"] - 100.0) < 5.0


def test_known_answer_16_beams():
    """tests/test_spectrum_maxima_rocm.hpp:196-233: 16 beams of sin(2 pi f t / fs) with
    f = 100 + 10 b Hz, fs 10 kHz, 1000 points, ONE_PEAK -> |refined f - f| < 10 Hz."""
    fs, n = 10000.0, 1000
    t = np.arange(n, dtype=np.float32)
    x = np.zeros((16, n), np.complex64)
    for b in range(16):
        f = np.float32(100.0 + 10.0 * b)
        x[b].real = np.sin(np.float32(2.0 * np.pi) * f * t / np.float32(fs))
    got = orc.one_two_peaks(orc.fft_fp32(x, 1024), 1024, 0, fs, False)
    assert got.shape == (16, 4)
    for b in range(16):
        assert abs(float(got[b, 0]["refined_frequency"]) - (100.0 + 10.0 * b)) < 10.0


def test_known_answer_spikes():
    """tests/test_spectrum_maxima_rocm.hpp:179-206: spikes at 50/120/200 on a 0.1 floor."""
    z = np.full((1, 1024), 0.1, np.complex64)
    z[0, [50, 120, 200]] = 5.0
    got, counts = orc.all_maxima(None, z, 1024, 1000.0)
    assert counts[0] == 3 and list(got[0, :3]["index"]) == [50, 120, 200]


def test_known_answer_magnitudes():
    """tests/test_complex_to_mag_phase_rocm.hpp:239-259: {3,4} -> 5, {0,0} -> 0."""
    z = np.array([3 + 4j, 0, 1e-6 + 1e-6j], np.complex64)
    m = orc.mag_rn(z)
    assert m[0] == 5.0 and m[1] == 0.0 and abs(m[2] - np.sqrt(2e-12)) < 1e-12


def test_tie_order_is_bit_reversed_thread_id():
    """Equal peaks at bins 10, 20, 30 of the left range: the reference's LDS tree
    returns 20 (bit-reversed-lid order), not the lowest bin."""
    z = np.zeros((1, 1024), np.complex64)
    z[0, [10, 20, 30]] = 5
    assert orc.one_two_peaks(z, 1024, 0, 1.0, False)[0, 0]["index"] == 20
    z = np.zeros((1, 1024), np.complex64)
    z[0, [100, 20, 30]] = 5
    assert orc.one_two_peaks(z, 1024, 0, 1.0, False)[0, 0]["index"] == 100


def test_noise_threshold_properties():
    """The histogram median is within one bucket (1/16 octave) of the exact median,
    and the 6-sigma threshold leaves ~1e-6 of pure-noise bins."""
    rng = np.random.default_rng(5)
    z = ((rng.standard_normal((4, 1 << 16)) + 1j * rng.standard_normal((4, 1 << 16))) / np.sqrt(2)).astype(np.complex64)
    mag = orc.mag_rn(z)
    med = orc.noise_threshold(mag, 1, 1 << 15, np.float32(1.0))
    exact = np.median(mag[:, 1:1 << 15], axis=1)
    assert np.all(np.abs(med / exact - 1) < 1 / 16)
    thr = orc.noise_threshold(mag, 1, 1 << 15, orc.noise_threshold_factor(6.0))
    frac = (mag[:, 1:1 << 15] > thr[:, None]).mean()
    assert frac < 1e-4


live = pytest.mark.skipif(not __import__("oracle.reference_lib", fromlist=["x"]).available(),
                          reason="oracle/_ref not built (reference sources absent)")


@live
@pytest.mark.parametrize("seed", range(3))
def test_live_reference_random_cases(seed):
    from oracle import reference_lib as ref
    rng = np.random.default_rng(1000 + seed)
    nfft = int(rng.choice([512, 1024, 3072]))
    z = (rng.integers(-2, 3, (3, nfft)) + 1j * rng.integers(-2, 3, (3, nfft))).astype(np.complex64)
    for two in (False, True):
        sr = int(rng.integers(2, nfft + 1))
        assert_mv_equal(orc.one_two_peaks(z, nfft, sr, 1e4, two).reshape(-1),
                        ref.post_peaks(z, nfft, sr, 1e4, two).reshape(-1))
    m = ref.compute_magnitudes(z)
    s, e = int(rng.integers(0, 40)), int(rng.integers(0, nfft + 5))
    r, rc = ref.all_maxima(m, z, nfft, 1.0, s, e, 200)
    o, oc = orc.all_maxima(m, z, nfft, 1.0, s, e, 200)
    np.testing.assert_array_equal(oc, rc)
    for b in range(3):
        n = min(int(rc[b]), r.shape[1])
        assert_mv_equal(o[b, :n], r[b, :n])
