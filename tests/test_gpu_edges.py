"""Edge cases of the path, through the C ABI: empty batches, single-sample
beams, the smallest and largest transform sizes, search windows at the
spectrum ends, capacity truncation, ragged uneven batches and argument
errors.  Results against the oracle as in the other suites."""
import ctypes as C

import numpy as np
import pytest

from oracle import spectrum_oracle as orc

pytestmark = pytest.mark.gpu


def _rand(beams, n, seed):
    rng = np.random.default_rng(seed)
    return ((rng.standard_normal((beams, n)) + 1j * rng.standard_normal((beams, n))) / np.sqrt(2)).astype(np.complex64)


def test_zero_beams_is_a_no_op_everywhere(spx, cuda):
    """beams == 0 / count == 0: SPX_OK and nothing touched, even with null pointers."""
    ctx = spx.default_context()
    ctx.bind_stream()
    L, h = spx.lib, ctx.h
    p = spx.peak_params(spx.PEAK_ALL)
    assert L.spx_fft(h, None, 0, 16, 16, 0, 0, 1.0, None) == 0
    assert L.spx_ifft(h, None, 0, 16, None) == 0
    assert L.spx_fft_r2c(h, None, 0, 16, 16, 0, 0, None) == 0
    assert L.spx_magnitude(h, None, None, 0, 1.0, 0) == 0
    assert L.spx_mag_phase(h, None, None, 0) == 0
    assert L.spx_peaks_one_two(h, None, 0, 1024, 0, 1.0, 0, None) == 0
    assert L.spx_all_maxima(h, None, None, 0, 1024, C.byref(p), None, None) == 0
    assert L.spx_fft_peaks(h, None, 0, 16, 16, 0, C.byref(p), None, None) == 0
    assert L.spx_fft_peaks_host(h, None, 0, 16, 16, 0, C.byref(p), None, None) == 0
    assert L.spx_synchronize(h) == 0


def test_single_sample_beams_and_tiny_sizes(spx, cuda):
    """n_point = 1 zero-padded to 2 .. 16 points, and nfft = n_point = 2, 3."""
    import torch
    for n_point, nfft in [(1, 2), (1, 16), (2, 2), (3, 3), (5, 6)]:
        x = _rand(4, n_point, n_point * 100 + nfft)
        got = spx.fft(torch.from_numpy(x).to(cuda), nfft).cpu().numpy()
        ref = orc.fft_fp64(x, nfft)
        assert np.abs(got - ref).max() <= 1e-5 * max(np.abs(ref).max(), 1e-30) + 1e-7


def test_maximum_single_pass_and_two_launch_sizes(spx, cuda):
    """262144 (largest single-pass size, cluster of 16) and 2^20 (two launches)."""
    import torch
    for nfft, n_point in [(262144, 200000), (1 << 20, 1 << 20)]:
        x = _rand(1, n_point, nfft)
        got = spx.fft(torch.from_numpy(x).to(cuda), nfft, window=spx.WINDOW_HANN).cpu().numpy()
        ref = orc.fft_fp64(x, nfft, orc.WINDOW_HANN)
        assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-5
    assert spx.fft_size_supported(1 << 21) and spx.fft_size_supported(1 << 22)
    assert not spx.fft_size_supported(1 << 29)


def test_more_beams_than_one_grid_dimension(spx, cuda):
    """65540 beams of a 32768-point transform (rows written to bin order by a
    transpose whose grid holds at most 65535 beams per launch): beams on both
    sides of the 65535 boundary equal pocketfft.  About 26 GB on the device."""
    import torch
    beams, n_point, nfft = 65540, 8, 32768
    x = _rand(beams, n_point, 3)
    got = spx.fft(torch.from_numpy(x).to(cuda), nfft, window=spx.WINDOW_NONE, out="mag2")
    torch.cuda.synchronize()
    for b in (0, 65534, 65535, 65536, beams - 1):
        ref = np.abs(orc.fft_fp32(x[b:b + 1], nfft)) ** 2
        row = got[b].cpu().numpy()
        assert np.abs(row - ref[0]).max() / ref.max() < 1e-5, b
    del got
    torch.cuda.empty_cache()


@pytest.mark.parametrize("start,end", [(1, 2), (1, 3), (0, 0), (1023, 1023), (1000, 4096), (2, 1024)])
def test_all_maxima_windows_at_the_ends(spx, cuda, start, end):
    """Empty / one-bin windows, end beyond nfft (clipped to nfft-1), windows
    touching bin 1 and bin nfft-2: counts and lists equal to the oracle."""
    import torch
    z = _rand(3, 2048, start + end)
    out, counts = spx.all_maxima(torch.from_numpy(z).to(cuda), sample_rate=1.0, search_start=start,
                                 search_end=end, max_per_beam=1000)
    ref, rc = orc.all_maxima(None, z, 2048, 1.0, start, end, 1000)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rc)
    got = spx.maxvalues_to_numpy(out)
    for b in range(3):
        n = min(int(rc[b]), ref.shape[1])
        np.testing.assert_array_equal(got[b, :n]["index"], ref[b, :n]["index"])


def test_all_maxima_capacity_truncation_keeps_untruncated_counts(spx, cuda):
    """More maxima than the capacity: the first `cap` in bin order are written,
    the count stays the untruncated total (all_maxima_pipeline_rocm.cpp:304-307)."""
    import torch
    z = _rand(2, 8192, 5)
    out, counts = spx.all_maxima(torch.from_numpy(z).to(cuda), sample_rate=1.0, max_per_beam=10)
    ref, rc = orc.all_maxima(None, z, 8192, 1.0, 0, 0, 10)
    c = counts.cpu().numpy().astype(np.uint32)
    np.testing.assert_array_equal(c, rc)
    assert (c > 10).all() and out.shape[1] == 10
    np.testing.assert_array_equal(spx.maxvalues_to_numpy(out)["index"], ref["index"])


def test_topk_fewer_maxima_than_k(spx, cuda):
    """A spectrum with 2 strict maxima and K = 8: count 2, remaining rows unused."""
    import torch
    f = np.full((1, 1024), 0.5, np.complex64)
    f[0, 100], f[0, 300] = 9.0, 7.0
    out, counts = spx.topk(torch.from_numpy(f).to(cuda), 8, sample_rate=1.0)
    assert int(counts[0]) == 2
    got = spx.maxvalues_to_numpy(out)[0, :2]
    np.testing.assert_array_equal(got["index"], [100, 300])


def test_ragged_uneven_batch_with_tiny_beams(spx, cuda):
    """Uneven batch including 1-, 2- and 3-sample beams and equal-length
    neighbours: single launch equals the per-size launches and the oracle."""
    import torch
    from spectrum_gb300.batch import Batch
    lengths = [1, 2, 3, 17, 1000, 1000, 4096, 16384, 20000, 65536]
    rng = np.random.default_rng(11)
    x = ((rng.standard_normal(sum(lengths)) + 1j * rng.standard_normal(sum(lengths)))).astype(np.complex64)
    xd = torch.from_numpy(x).to(cuda)
    # a peak search needs nfft >= 3: the tiny beams are zero-padded to 4 points
    nffts = [max(4, spx.next_smooth23(n)) for n in lengths]
    b = Batch(lengths, nffts=nffts, window=0, k=4, sample_rate=1.0)
    o1, c1 = [t.clone() for t in b.run(xd)]
    o2, c2 = [t.clone() for t in b.run_per_size(xd)]
    np.testing.assert_array_equal(c1.cpu().numpy(), c2.cpu().numpy())
    g1, g2 = spx.maxvalues_to_numpy(o1), spx.maxvalues_to_numpy(o2)
    off = 0
    for i, (n, nfft) in enumerate(zip(lengths, nffts)):
        beam = x[off:off + n][None]
        off += n
        cnt = int(c1[i])
        np.testing.assert_array_equal(g1[i, :cnt]["index"], g2[i, :cnt]["index"])
        ref, rc = orc.topk(None, spx.fft(torch.from_numpy(beam).to(cuda), nfft).cpu().numpy(), nfft, 1.0, 4)
        assert cnt == int(rc[0])
        np.testing.assert_array_equal(g1[i, :cnt]["index"], ref[0, :cnt]["index"])


def test_argument_errors_are_invalid_argument(spx, cuda):
    import torch
    x = torch.zeros((2, 64), dtype=torch.complex64, device=cuda)
    with pytest.raises(ValueError):
        spx.fft(x, 32)                       # nfft < n_point
    with pytest.raises(ValueError):
        spx.fft(x, (1 << 27) + 1)            # no direct plan and too long for Bluestein
    with pytest.raises(ValueError):
        spx.topk(x, 33)                      # K > 32
    with pytest.raises(ValueError):
        spx.topk(x, 0)
    with pytest.raises(ValueError):
        spx.all_maxima(x, thresh_sigma=-1.0)
    with pytest.raises(ValueError):
        spx.fft_peaks(x, 64, mode=7)


@pytest.mark.parametrize("nfft,n_point,start,end,sigma", [
    (131072, 65536, 1, 2, 0.0),              # one bin
    (131072, 65536, 65535, 65536, 0.0),      # one bin at the default end
    (131072, 65536, 131060, 131071, 0.0),    # last bins; end = nfft - 1
    (131072, 65536, 100, 300, 1.0),          # narrower than one CTA's share of the maxima kernel
    (131072, 100000, 7, 200000, 2.0),        # end beyond nfft: clipped to nfft - 1
    (65536, 65536, 3, 65533, 0.5),           # groups of 4 CTAs, many maxima above the threshold
    (39366, 39000, 11, 39360, 6.0),          # 3-smooth size (cluster path), wide window
])
def test_large_fused_search_window_edges(spx, cuda, nfft, n_point, start, end, sigma):
    """spx_fft_peaks for nfft > 16384 (the FFT writes only the window's bins,
    then the maxima kernel): counts and records equal to the oracle on the
    spectrum spx_fft returns, for windows at the ends and of every width."""
    import torch
    x = _rand(2, n_point, nfft + start)
    xd = torch.from_numpy(x).to(cuda)
    spec = spx.fft(xd, nfft, window=spx.WINDOW_HANN).cpu().numpy()
    out, counts = spx.fft_peaks(xd, nfft, spx.WINDOW_HANN, spx.PEAK_ALL, sample_rate=1.0, refine=1,
                                thresh_sigma=sigma, search_start=start, search_end=end)
    ref, rc = orc.all_maxima(None, spec, nfft, 1.0, start, end, refine=1, thresh_sigma=sigma)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rc)
    got = spx.maxvalues_to_numpy(out)
    for b in range(2):
        n = min(int(rc[b]), ref.shape[1])
        for f in ["index", "real", "imag", "magnitude", "freq_offset", "refined_frequency"]:
            np.testing.assert_array_equal(got[b, :n][f], ref[b, :n][f], err_msg=f"beam {b} field {f}")
