"""GPU parity of the peak search against the oracle on the SAME spectrum.

Bit-exact: index, real, imag, magnitude, freq_offset, refined_frequency and
the per-beam counts.  phase (atan2 in degrees) within 1e-4 degree, the only
field computed by a transcendental whose last bit differs between CUDA and
the host libm.
"""
import numpy as np
import pytest

from oracle import spectrum_oracle as orc

pytestmark = pytest.mark.gpu

EXACT = ["index", "real", "imag", "magnitude", "freq_offset", "refined_frequency", "pad"]


def assert_maxvalues_equal(got, ref, n=None):
    if n is not None:
        got, ref = got[:n], ref[:n]
    for f in EXACT:
        np.testing.assert_array_equal(got[f], ref[f], err_msg=f"field {f}")
    np.testing.assert_allclose(got["phase"], ref["phase"], rtol=0, atol=1e-4, err_msg="phase")


def _noise_spectrum(beams, nfft, seed, tones=0):
    rng = np.random.default_rng(seed)
    z = (rng.standard_normal((beams, nfft)) + 1j * rng.standard_normal((beams, nfft))).astype(np.complex64)
    for b in range(beams):
        for _ in range(tones):
            k = rng.integers(2, nfft - 2)
            z[b, k] += np.complex64(rng.uniform(20, 200) * np.exp(1j * rng.uniform(0, 6.28)))
            z[b, k + 1] += np.complex64(rng.uniform(5, 50))
    return z


def _tie_spectrum(beams, nfft, seed):
    """Small-integer spectra: many exactly equal magnitudes and plateaus."""
    rng = np.random.default_rng(seed)
    return (rng.integers(-3, 4, (beams, nfft)) + 1j * rng.integers(-3, 4, (beams, nfft))).astype(np.complex64)


def _dev(a, cuda):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


# ---- ONE_PEAK / TWO_PEAKS ------------------------------------------------------
@pytest.mark.parametrize("nfft,search_range", [(1024, 0), (1024, 1024), (4096, 300), (2048, 2), (8192, 4096)])
@pytest.mark.parametrize("kind", ["noise", "ties"])
@pytest.mark.parametrize("two", [False, True])
def test_one_two_peaks(spx, cuda, nfft, search_range, kind, two):
    z = _noise_spectrum(5, nfft, nfft, tones=2) if kind == "noise" else _tie_spectrum(5, nfft, nfft)
    got = spx.maxvalues_to_numpy(spx.peaks_one_two(_dev(z, cuda), search_range, 10000.0, two))
    ref = orc.one_two_peaks(z, nfft, search_range, 10000.0, two)
    assert_maxvalues_equal(got, ref)


def test_one_peak_known_answer(spx, cuda):
    """100 Hz sine, fs 10 kHz, 1000 points -> nFFT 1024: |f - 100| < 5 Hz
    (tests/test_spectrum_maxima_rocm.hpp:98-126)."""
    import torch
    n, fs = 1000, 10000.0
    t = np.arange(n)
    x = np.exp(2j * np.pi * 100.0 * t / fs).astype(np.complex64)[None].repeat(4, 0)
    spec = spx.fft(_dev(x, cuda), 1024)
    got = spx.maxvalues_to_numpy(spx.peaks_one_two(spec, 0, fs, False))
    assert np.all(np.abs(got[:, 0]["refined_frequency"] - 100.0) < 5.0)


# ---- ALL_MAXIMA --------------------------------------------------------------------
ALL_CASES = [
    # nfft, beams, start, end, max_per_beam, kind
    (1024, 3, 0, 0, 1000, "noise"),
    (1024, 3, 0, 0, 1000, "ties"),
    (16384, 2, 0, 0, 1000, "noise"),       # several tiles, capacity-truncated
    (16384, 2, 0, 0, 100000, "noise"),     # several tiles, no truncation
    (131072, 4, 0, 0, 1 << 20, "noise"),   # 32 tiles per beam
    (4096, 2, 5, 4096, 50, "ties"),        # end >= nfft -> nfft - 1
    (4096, 2, 3000, 100, 1000, "noise"),   # empty window (end < start)
    (2048, 1, 1, 3, 1000, "noise"),        # tiny window
    (524288, 1, 0, 262145, 1000, "noise"),  # 262144 bins: the longest window of the cluster kernel
    (1 << 20, 1, 0, (1 << 20) - 1, 1000, "noise"),  # longer: the look-back kernel
]


@pytest.mark.parametrize("nfft,beams,start,end,cap,kind", ALL_CASES)
@pytest.mark.parametrize("with_mag", [True, False])
def test_all_maxima_reference_semantics(spx, cuda, nfft, beams, start, end, cap, kind, with_mag):
    z = _noise_spectrum(beams, nfft, nfft + start) if kind == "noise" else _tie_spectrum(beams, nfft, nfft)
    mag = orc.mag_rn(z)
    out, counts = spx.all_maxima(_dev(z, cuda), _dev(mag, cuda) if with_mag else None, 48000.0,
                                 start, end, cap)
    got = spx.maxvalues_to_numpy(out)
    counts = counts.cpu().numpy().astype(np.uint32)
    ref, rcounts = orc.all_maxima(mag, z, nfft, 48000.0, start, end, cap)
    np.testing.assert_array_equal(counts, rcounts)
    for b in range(beams):
        assert_maxvalues_equal(got[b], ref[b], n=min(int(rcounts[b]), ref.shape[1]))


def test_all_maxima_spikes_known_answer(spx, cuda):
    """Spikes at bins 50/120/200 on a 0.1 floor are found
    (tests/test_spectrum_maxima_rocm.hpp:179-206)."""
    nfft = 1024
    z = np.full((2, nfft), 0.1, np.complex64)
    for k in (50, 120, 200):
        z[:, k] = 5.0
    out, counts = spx.all_maxima(_dev(z, cuda), None, 1000.0)
    got = spx.maxvalues_to_numpy(out)
    assert list(counts.cpu().numpy()) == [3, 3]
    assert list(got[0, :3]["index"]) == [50, 120, 200]


@pytest.mark.parametrize("refine", [0, 1])
@pytest.mark.parametrize("sigma", [0.0, 6.0, 3.0])
def test_all_maxima_threshold_and_refine(spx, cuda, refine, sigma):
    nfft = 8192
    z = _noise_spectrum(4, nfft, 11, tones=6)
    out, counts = spx.all_maxima(_dev(z, cuda), None, 1000.0, 0, 0, 1000, refine, sigma)
    got = spx.maxvalues_to_numpy(out)
    counts = counts.cpu().numpy().astype(np.uint32)
    ref, rcounts = orc.all_maxima(None, z, nfft, 1000.0, 0, 0, 1000, refine, sigma)
    np.testing.assert_array_equal(counts, rcounts)
    for b in range(4):
        assert_maxvalues_equal(got[b], ref[b], n=int(rcounts[b]))
    if sigma == 6.0:  # planted lines inside [1, nfft/2) survive, noise maxima do not
        assert (rcounts >= 1).all() and (rcounts < 20).all()


@pytest.mark.parametrize("nfft,end", [(524288, 262145), (1 << 20, (1 << 20) - 1)])
def test_all_maxima_threshold_at_window_limits(spx, cuda, nfft, end):
    """Thresholded search at 262144 bins (cluster kernel, 32768 bins per CTA)
    and beyond (histogram/select kernels + look-back kernel): oracle lists."""
    z = _noise_spectrum(1, nfft, 5, tones=30)
    out, counts = spx.all_maxima(_dev(z, cuda), None, 1000.0, 1, end, 1000, 1, 3.0)
    ref, rcounts = orc.all_maxima(None, z, nfft, 1000.0, 1, end, 1000, 1, 3.0)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rcounts)
    assert_maxvalues_equal(spx.maxvalues_to_numpy(out)[0], ref[0], n=min(int(rcounts[0]), ref.shape[1]))


# ---- TOP-K -----------------------------------------------------------------------
@pytest.mark.parametrize("nfft,k", [(4096, 5), (4096, 1), (1024, 32), (131072, 8), (2048, 8)])
@pytest.mark.parametrize("kind", ["noise", "ties"])
def test_topk(spx, cuda, nfft, k, kind):
    z = _noise_spectrum(3, nfft, k, tones=3) if kind == "noise" else _tie_spectrum(3, nfft, k)
    out, counts = spx.topk(_dev(z, cuda), k, None, 4096.0)
    got = spx.maxvalues_to_numpy(out)
    ref, rcounts = orc.topk(None, z, nfft, 4096.0, k)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rcounts)
    for b in range(3):
        assert_maxvalues_equal(got[b], ref[b], n=int(rcounts[b]))


@pytest.mark.parametrize("nfft,start,end,k", [
    (4096, 37, 1000, 5),        # unaligned window over several warp steps
    (4096, 1, 20, 8),           # window narrower than one run of 32 bins
    (8192, 3000, 8191, 16),     # window ending at the last bin
    (65536, 5, 40000, 32),      # many 2048-bin steps, K = 32
])
@pytest.mark.parametrize("with_mag", [False, True])
def test_topk_windows_and_magnitude_input(spx, cuda, nfft, start, end, k, with_mag):
    """spx_topk over search windows of any start and length, including one
    ending at the last bin, and over a caller's magnitude array (independent
    of the spectrum, so the kernel must take |X| from it): the oracle's lists."""
    z = _noise_spectrum(3, nfft, 17, tones=6)
    mag = np.random.default_rng(5).random((3, nfft), dtype=np.float32) if with_mag else None
    out, counts = spx.topk(_dev(z, cuda), k, None if mag is None else _dev(mag, cuda), 1000.0,
                           search_start=start, search_end=end)
    ref, rcounts = orc.topk(mag, z, nfft, 1000.0, k, start, end)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rcounts)
    got = spx.maxvalues_to_numpy(out)
    for b in range(3):
        assert_maxvalues_equal(got[b], ref[b], n=int(rcounts[b]))


def test_topk_with_threshold(spx, cuda):
    z = _noise_spectrum(3, 8192, 5, tones=4)
    out, counts = spx.topk(_dev(z, cuda), 16, None, 1.0, thresh_sigma=6.0)
    ref, rcounts = orc.topk(None, z, 8192, 1.0, 16, thresh_sigma=6.0)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rcounts)
    got = spx.maxvalues_to_numpy(out)
    for b in range(3):
        assert_maxvalues_equal(got[b], ref[b], n=int(rcounts[b]))


# ---- composed / fused raw samples -> peaks ----------------------------------------
@pytest.mark.parametrize("mode", ["one", "two", "all", "topk"])
def test_fft_peaks_matches_oracle_on_same_spectrum(spx, cuda, mode):
    from spectrum_gb300 import synth
    bs = synth.workload_small(seed=3)
    x = synth.synth_numpy(bs)
    nfft, fs = 4096, 1.0
    xd = _dev(x, cuda)
    spec = spx.fft(xd, nfft, window=spx.WINDOW_HANN).cpu().numpy()
    pm = {"one": spx.PEAK_ONE, "two": spx.PEAK_TWO, "all": spx.PEAK_ALL, "topk": spx.PEAK_TOPK}[mode]
    kw = dict(sample_rate=fs, refine=1, thresh_sigma=6.0 if mode == "all" else 0.0,
              max_per_beam=5 if mode == "topk" else 1000, search_range=nfft)
    out, counts = spx.fft_peaks(xd, nfft, spx.WINDOW_HANN, pm, **kw)
    got = spx.maxvalues_to_numpy(out)
    if mode in ("one", "two"):
        ref = orc.one_two_peaks(spec, nfft, nfft, fs, mode == "two")
        assert_maxvalues_equal(got, ref)
    elif mode == "all":
        ref, rc = orc.all_maxima(None, spec, nfft, fs, refine=1, thresh_sigma=6.0)
        np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rc)
        for b in range(len(rc)):
            assert_maxvalues_equal(got[b], ref[b], n=int(rc[b]))
    else:
        ref, rc = orc.topk(None, spec, nfft, fs, 5)
        np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rc)
        for b in range(len(rc)):
            assert_maxvalues_equal(got[b], ref[b], n=int(rc[b]))
        # the three tones of every beam are the top-3 (sigma 0.01 noise)
        for b in range(bs.beams):
            f_true = np.sort(bs.freqs[b])
            f_got = np.sort(got[b, :3]["refined_frequency"])
            assert np.all(np.abs(f_got - f_true) < 1.0 / nfft)


def test_status_word_clean_after_runs(spx, cuda):
    """No bounded device wait expired during the tests above."""
    spx.default_context().synchronize()


def test_bounded_wait_times_out_and_context_stays_usable(spx, cuda):
    """A look-back wait on a status word nothing publishes gives up after its
    1 s bound: the call reports SPX_ERR_TIMEOUT, the error word is cleared,
    and the same context then runs an all-maxima search correctly."""
    import time

    import torch
    ctx = spx.default_context()
    ctx.bind_stream()
    t0 = time.perf_counter()
    st = spx.lib.spx_selftest_wait_timeout(ctx.h)
    dt = time.perf_counter() - t0
    assert st == spx._capi.SPX_ERR_TIMEOUT
    assert 0.9 < dt < 30.0
    assert b"bounded device-side wait" in spx.lib.spx_last_error(ctx.h)
    assert spx.lib.spx_synchronize(ctx.h) == spx._capi.SPX_OK
    rng = np.random.default_rng(3)
    z = (rng.standard_normal((4, 8192)) + 1j * rng.standard_normal((4, 8192))).astype(np.complex64)
    out, counts = spx.all_maxima(torch.from_numpy(z).to(cuda), sample_rate=1.0)
    ref, rc = orc.all_maxima(None, z, 8192, 1.0)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rc)


def test_group_barrier_wait_times_out_and_context_stays_usable(spx, cuda):
    """The per-beam group barrier of the large fused transform gives up after
    its 1 s bound when an arrival never comes: SPX_ERR_TIMEOUT, then the same
    context runs the large fused search (which uses that barrier) correctly."""
    import time

    import torch
    from spectrum_gb300 import synth
    ctx = spx.default_context()
    ctx.bind_stream()
    t0 = time.perf_counter()
    st = spx.lib.spx_selftest_group_wait_timeout(ctx.h)
    dt = time.perf_counter() - t0
    assert st == spx._capi.SPX_ERR_TIMEOUT
    assert 0.9 < dt < 30.0
    assert spx.lib.spx_synchronize(ctx.h) == spx._capi.SPX_OK
    bs = synth.make_beams([65536] * 3, tones=(1, 8), snr_db=(10.0, 40.0), seed=5)
    x = synth.synth_numpy(bs)
    xd = torch.from_numpy(x).to(cuda)
    spec = spx.fft(xd, 131072, window=spx.WINDOW_HANN).cpu().numpy()
    out, counts = spx.fft_peaks(xd, 131072, spx.WINDOW_HANN, spx.PEAK_ALL, sample_rate=1.0, thresh_sigma=6.0)
    ref, rc = orc.all_maxima(None, spec, 131072, 1.0, thresh_sigma=6.0)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rc)
    np.testing.assert_array_equal(spx.maxvalues_to_numpy(out)[0, :int(rc[0])]["index"], ref[0, :int(rc[0])]["index"])
