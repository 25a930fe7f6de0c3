"""GPU checks of the Python mirror of the reference's ``dsp_spectrum`` module
(spectrum_gb300.dsp_spectrum): shapes and keys of its results as the
pybind11 classes return them, and values against the oracle on the same
spectrum (bit-exact peaks, FFT within 1e-5 of pocketfft)."""
import numpy as np
import pytest

from oracle import spectrum_oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dsp(spx):
    from spectrum_gb300 import dsp_spectrum
    return dsp_spectrum


@pytest.fixture(scope="module")
def ctx(dsp, cuda):
    return dsp.ROCmGPUContext(device_index=0)


def _tone(f, fs, n, beams=1, real=False, seed=0):
    t = np.arange(n)
    x = np.exp(2j * np.pi * f * t / fs) if not real else np.sin(2 * np.pi * f * t / fs) + 0j
    rng = np.random.default_rng(seed)
    x = np.tile(x, (beams, 1)) + 0.01 * (rng.standard_normal((beams, n)) + 1j * rng.standard_normal((beams, n)))
    return x.astype(np.complex64)


def test_context(ctx):
    assert ctx.device_index == 0
    assert "GB300" in ctx.device_name or ctx.device_name


def test_fft_processor_complex_and_mag_phase(dsp, ctx):
    fft = dsp.FFTProcessorROCm(ctx)
    x = _tone(100.0, 1000.0, 1000, beams=3)
    spec = fft.process_complex(x, sample_rate=1000.0)
    assert spec.shape == (3, 1024) and spec.dtype == np.complex64 and fft.nfft == 1024
    ref = orc.fft_fp32(x, 1024)
    assert np.abs(spec - ref).max() / np.abs(ref).max() < 1e-5
    one = fft.process_complex(x[0], sample_rate=1000.0)
    assert one.shape == (1024,)
    np.testing.assert_array_equal(one, spec[0])
    mp = fft.process_mag_phase(x, sample_rate=1000.0)
    assert set(mp) == {"magnitude", "phase", "frequency", "nFFT", "sample_rate"}
    assert mp["magnitude"].shape == (3, 1024) and mp["nFFT"] == 1024
    np.testing.assert_array_equal(mp["magnitude"], orc.mag_rn(spec))
    np.testing.assert_allclose(mp["phase"], np.angle(spec), atol=4e-6)
    np.testing.assert_array_equal(mp["frequency"][1], np.arange(1024, dtype=np.float32) * np.float32(1000.0 / 1024))
    mp1 = fft.process_mag_phase(x[:1], sample_rate=1000.0, include_freq=False)
    assert "frequency" not in mp1 and mp1["magnitude"].shape == (1024,)
    prof = fft.get_profiling()
    assert set(prof) == {"upload_ms", "fft_ms", "post_processing_ms", "download_ms", "total_ms"}
    assert prof["fft_ms"] > 0


def test_complex_to_mag(dsp, ctx):
    c = dsp.ComplexToMagROCm(ctx)
    x = _tone(7.0, 64.0, 512, beams=4)
    for norm, inv in ((1.0, 1.0), (0.0, 1.0), (-1.0, np.float32(1.0) / np.float32(512)), (2.5, 2.5)):
        m = c.process_magnitude(x, beam_count=4, norm_coeff=norm)
        assert m.shape == (4, 512)
        np.testing.assert_array_equal(m, orc.magnitude(x, np.float32(inv)))
    assert c.process_magnitude(x[0]).shape == (512,)
    with pytest.raises(ValueError):
        c.process_magnitude(x.reshape(-1)[:1001], beam_count=4)


def test_maxima_finder_process_one_peak(dsp, ctx, spx):
    """100 Hz at fs 10 kHz, 1000 points (tests/test_spectrum_maxima_rocm.hpp:99-124)
    within 5 Hz, and bit-exact against the oracle's post_kernel_one_peak."""
    import torch
    f = dsp.SpectrumMaximaFinderROCm(ctx)
    assert not f.is_initialized()
    x = _tone(100.0, 10000.0, 1000, beams=4, real=True)
    res = f.process(x, n_point=1000, sample_rate=10000.0)
    assert isinstance(res, list) and len(res) == 4
    assert set(res[0]) == {"antenna_id", "freq_hz", "magnitude", "phase", "index", "freq_offset"}
    for r in res:
        assert abs(r["freq_hz"] - 100.0) < 5.0
    spec = spx.fft(torch.from_numpy(x).cuda(), 1024).cpu().numpy()
    ref = orc.one_two_peaks(spec, 1024, 256, 10000.0, two=False)
    for b, r in enumerate(res):
        assert r["index"] == ref[b, 0]["index"]
        assert np.float32(r["freq_hz"]) == ref[b, 0]["refined_frequency"]
        assert np.float32(r["freq_offset"]) == ref[b, 0]["freq_offset"]
    single = f.process(x[0], n_point=1000, sample_rate=10000.0)
    assert isinstance(single, dict) and single["antenna_id"] == 0
    p = f.get_params()
    assert p["nFFT"] == 1024 and p["n_point"] == 1000 and f.is_initialized()


def test_maxima_finder_all_maxima_known_answer(dsp, ctx):
    """A 0.1 floor with bins 50 / 120 / 200 (tests/test_spectrum_maxima_rocm.hpp:182-185)."""
    f = dsp.SpectrumMaximaFinderROCm(ctx)
    fft = np.full(1024, 0.1, np.complex64)
    fft[50], fft[120], fft[200] = 100, 80, 60
    r = f.find_all_maxima(fft, nFFT=1024, sample_rate=1000.0)
    assert isinstance(r, dict) and r["num_maxima"] == 3
    np.testing.assert_array_equal(r["positions"], [50, 120, 200])
    np.testing.assert_array_equal(r["magnitudes"], np.float32([100, 80, 60]))
    np.testing.assert_array_equal(r["frequencies"], np.float32([50, 120, 200]) * np.float32(1000.0 / 1024))


def test_maxima_finder_all_maxima_from_signal_matches_oracle(dsp, ctx, spx):
    import torch
    f = dsp.SpectrumMaximaFinderROCm(ctx)
    x = _tone(50.0, 1000.0, 1000, beams=3, real=True, seed=5)
    res = f.find_all_maxima_from_signal(x, n_point=1000, sample_rate=1000.0, repeat_count=2)
    assert len(res) == 3
    spec = spx.fft(torch.from_numpy(x).cuda(), 2048).cpu().numpy()
    ref, rc = orc.all_maxima(None, spec, 2048, 1000.0)
    for b, r in enumerate(res):
        n = min(int(rc[b]), ref.shape[1])
        assert r["num_maxima"] == n
        np.testing.assert_array_equal(r["positions"], ref[b, :n]["index"])
        np.testing.assert_array_equal(r["magnitudes"], ref[b, :n]["magnitude"])
        np.testing.assert_array_equal(r["frequencies"], ref[b, :n]["refined_frequency"])
    # the same spectra through find_all_maxima
    res2 = f.find_all_maxima(spec, nFFT=2048, sample_rate=1000.0)
    for r, r2 in zip(res, res2):
        np.testing.assert_array_equal(r["positions"], r2["positions"])


def test_maxima_finder_rejects_bad_input(dsp, ctx):
    f = dsp.SpectrumMaximaFinderROCm(ctx)
    with pytest.raises(ValueError):
        f.process(np.zeros(999, np.complex64), n_point=1000, sample_rate=1.0)
    with pytest.raises(ValueError):
        f.find_all_maxima(np.zeros(100, np.complex64), nFFT=1024, sample_rate=1.0)
