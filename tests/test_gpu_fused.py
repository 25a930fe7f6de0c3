"""GPU parity of the fused raw-samples -> peaks kernel (spx_fft_peaks).

The oracle runs on the spectrum spx_fft returns for the same samples; the
fused kernel never writes that spectrum, so equal peak lists (bit-exact
indices, counts and fields; phase within 1e-4 degree) also show the fused
transform computes the same bits as the plain one.
"""
import numpy as np
import pytest

from oracle import spectrum_oracle as orc

pytestmark = pytest.mark.gpu

EXACT = ["index", "real", "imag", "magnitude", "freq_offset", "refined_frequency", "pad"]


def assert_rows_equal(got, ref, counts):
    for b in range(len(counts)):
        n = min(int(counts[b]), ref.shape[1])
        for f in EXACT:
            np.testing.assert_array_equal(got[b, :n][f], ref[b, :n][f], err_msg=f"beam {b} field {f}")
        np.testing.assert_allclose(got[b, :n]["phase"], ref[b, :n]["phase"], atol=1e-4, rtol=0)


def _beams(n_beams, n_point, seed, tones=(1, 16)):
    from spectrum_gb300 import synth
    bs = synth.make_beams([n_point] * n_beams, tones=tones, snr_db=(0.0, 40.0), seed=seed)
    return synth.synth_numpy(bs)


# nfft -> cluster size: 4096 (1), 16384 (1), 17496 (3), 20736 (3), 32768 (4), 39366 (6),
# 65536 (8), 59049 (9), 78732 (12), 104976 (16), 131072 (16)
ALL_CASES = [(4096, 4096, 6), (16384, 16384, 4), (17496, 17000, 3), (32768, 20000, 3),
             (39366, 39366, 2), (65536, 65536, 2), (59049, 59049, 2), (78732, 78000, 2),
             (104976, 100000, 2), (131072, 65536, 4)]


@pytest.mark.parametrize("nfft,n_point,beams", ALL_CASES)
@pytest.mark.parametrize("refine", [0, 1])
def test_fused_all_maxima_thresholded(spx, cuda, nfft, n_point, beams, refine):
    import torch
    x = _beams(beams, n_point, nfft + refine)
    xd = torch.from_numpy(x).to(cuda)
    spec = spx.fft(xd, nfft, window=spx.WINDOW_HANN).cpu().numpy()
    out, counts = spx.fft_peaks(xd, nfft, spx.WINDOW_HANN, spx.PEAK_ALL, sample_rate=48000.0,
                                refine=refine, thresh_sigma=6.0)
    ref, rc = orc.all_maxima(None, spec, nfft, 48000.0, refine=refine, thresh_sigma=6.0)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rc)
    assert_rows_equal(spx.maxvalues_to_numpy(out), ref, rc)
    assert rc.min() >= 1


@pytest.mark.parametrize("nfft,n_point,sigma,start,end", [(131072, 65536, 0.5, 0, 0), (65536, 65536, 1.0, 0, 0),
                                                         (131072, 100000, 2.0, 5000, 120000),
                                                         (39366, 39366, 0.25, 3, 39000)])
def test_fused_cluster_many_hot_bins(spx, cuda, nfft, n_point, sigma, start, end):
    """Low thresholds: thousands of bins above the threshold's bucket, so the
    cluster epilogue takes its bitmap path; lists equal to the oracle's."""
    import torch
    x = _beams(3, n_point, nfft + int(sigma * 8))
    xd = torch.from_numpy(x).to(cuda)
    spec = spx.fft(xd, nfft, window=spx.WINDOW_HANN).cpu().numpy()
    out, counts = spx.fft_peaks(xd, nfft, spx.WINDOW_HANN, spx.PEAK_ALL, sample_rate=48000.0, refine=1,
                                thresh_sigma=sigma, search_start=start, search_end=end)
    ref, rc = orc.all_maxima(None, spec, nfft, 48000.0, start, end, refine=1, thresh_sigma=sigma)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rc)
    assert_rows_equal(spx.maxvalues_to_numpy(out), ref, rc)
    assert rc.min() > 1024 // 8


@pytest.mark.parametrize("nfft,start,end,cap", [(4096, 0, 0, 1000), (8192, 100, 3000, 64), (2048, 1, 2047, 10)])
def test_fused_all_maxima_reference_semantics_single_cta(spx, cuda, nfft, start, end, cap):
    """No threshold (every strict local maximum), C = 1: still one fused launch."""
    import torch
    x = _beams(3, nfft, 7)
    xd = torch.from_numpy(x).to(cuda)
    spec = spx.fft(xd, nfft).cpu().numpy()
    out, counts = spx.fft_peaks(xd, nfft, spx.WINDOW_NONE, spx.PEAK_ALL, sample_rate=1.0,
                                search_start=start, search_end=end, max_per_beam=cap)
    ref, rc = orc.all_maxima(None, spec, nfft, 1.0, start, end, cap)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rc)
    assert_rows_equal(spx.maxvalues_to_numpy(out), ref, rc)


@pytest.mark.parametrize("nfft,k,sigma", [(4096, 5, 0.0), (8192, 8, 6.0), (1024, 32, 0.0), (16384, 8, 3.0)])
def test_fused_topk_single_cta(spx, cuda, nfft, k, sigma):
    import torch
    x = _beams(4, nfft, k)
    xd = torch.from_numpy(x).to(cuda)
    spec = spx.fft(xd, nfft, window=spx.WINDOW_HANN).cpu().numpy()
    out, counts = spx.fft_peaks(xd, nfft, spx.WINDOW_HANN, spx.PEAK_TOPK, sample_rate=1.0,
                                max_per_beam=k, refine=1, thresh_sigma=sigma)
    ref, rc = orc.topk(None, spec, nfft, 1.0, k, thresh_sigma=sigma)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rc)
    assert_rows_equal(spx.maxvalues_to_numpy(out), ref, rc)


@pytest.mark.parametrize("nfft,beams,mode,k,sigma", [(4096, 600, "all", 1000, 6.0), (8192, 1100, "topk", 8, 0.0),
                                                     (16384, 600, "topk", 4, 3.0)])
def test_fft_peaks_beyond_the_single_cta_limit(spx, cuda, nfft, beams, mode, k, sigma):
    """spx_fft_peaks calls too large for the single-CTA fused kernel to pay
    (the spectrum goes to device memory, then the search kernel): the same
    counts and records as the oracle on spx_fft's spectrum."""
    import torch
    x = _beams(beams, nfft, nfft + beams, tones=(1, 4))
    xd = torch.from_numpy(x).to(cuda)
    spec = spx.fft(xd, nfft, window=spx.WINDOW_HANN).cpu().numpy()
    pm = spx.PEAK_ALL if mode == "all" else spx.PEAK_TOPK
    out, counts = spx.fft_peaks(xd, nfft, spx.WINDOW_HANN, pm, sample_rate=1.0, max_per_beam=k, refine=1,
                                thresh_sigma=sigma)
    if mode == "all":
        ref, rc = orc.all_maxima(None, spec, nfft, 1.0, 0, 0, k, refine=1, thresh_sigma=sigma)
    else:
        ref, rc = orc.topk(None, spec, nfft, 1.0, k, thresh_sigma=sigma)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rc)
    assert_rows_equal(spx.maxvalues_to_numpy(out), ref, rc)


def test_fused_large_workload_properties(spx, cuda):
    """The benchmark workload's full size (256 x 65536 -> 131072): bins
    ascend, counts fit the capacity, every one of the 256 beams matches the
    oracle exactly on the same spectra, and the planted tones are found."""
    import torch
    from spectrum_gb300 import synth
    bs = synth.workload_large(seed=1, beams=256)
    xd = synth.synth_torch(bs, device=cuda)
    nfft = 131072
    out, counts = spx.fft_peaks(xd, nfft, spx.WINDOW_HANN, spx.PEAK_ALL, sample_rate=1.0,
                                refine=1, thresh_sigma=6.0)
    got = spx.maxvalues_to_numpy(out)
    counts = counts.cpu().numpy().astype(np.uint32)
    assert (counts >= 1).all() and (counts <= out.shape[1]).all()
    for b in range(256):
        idx = got[b, : counts[b]]["index"]
        assert np.all(np.diff(idx.astype(np.int64)) > 0)
    sample = list(range(256))
    spec = spx.fft(xd, nfft, window=spx.WINDOW_HANN).cpu().numpy()
    ref, rc = orc.all_maxima(None, spec, nfft, 1.0, refine=1, thresh_sigma=6.0)
    np.testing.assert_array_equal(counts[sample], rc)
    assert_rows_equal(got[sample], ref, rc)
    # every planted tone (freq in [0, 0.5) cycles/sample) is found within one bin
    for j, b in enumerate(sample):
        f = got[b, : counts[b]]["refined_frequency"]
        fr = np.asarray(bs.freqs[b])
        for ft, a in zip(bs.freqs[b], bs.amps[b]):
            others = np.abs(fr - ft)
            isolated = np.sort(others)[1] > 16.0 / nfft if len(fr) > 1 else True
            if a >= 0.5 * max(bs.amps[b]) and isolated:
                assert np.min(np.abs(f - ft)) < 2.0 / nfft


@pytest.mark.parametrize("nfft,n_point,beams,mode,k,sigma,pinned", [
    (131072, 65536, 70, "all", 1000, 6.0, True),    # 35 MiB mapped: read in place
    (131072, 65536, 137, "all", 1000, 6.0, True),   # more beams than resident beam groups
    (65536, 60000, 250, "all", 1000, 3.0, True),    # 114 MiB: 8 uploaded chunks, groups of 4 CTAs
    (4096, 4096, 4100, "topk", 5, 0.0, True),      # 128 MiB: 9 chunks, input and output slots reused
    (4096, 4096, 1300, "topk", 5, 0.0, True),      # 40 MiB mapped: read in place
    (4096, 4000, 1100, "one", 0, 0.0, False),      # pageable numpy input, ONE_PEAK (no counts)
])
def test_fft_peaks_host_matches_device_path(spx, cuda, nfft, n_point, beams, mode, k, sigma, pinned):
    """spx_fft_peaks_host (host in, host out; mapped input read in place or,
    above 112 MiB, uploaded in chunks that overlap the compute) returns
    exactly what spx_fft_peaks returns on the same samples, with the peaks
    copied back or written in place into page-locked outputs."""
    import torch
    from spectrum_gb300 import synth
    bs = synth.make_beams([n_point] * beams, tones=(1, 8), snr_db=(0.0, 40.0), seed=nfft + beams)
    xd = synth.synth_torch(bs, device=cuda)
    m = {"all": spx.PEAK_ALL, "topk": spx.PEAK_TOPK, "one": spx.PEAK_ONE}[mode]
    kw = dict(sample_rate=1000.0, refine=spx.REFINE_PARABOLIC, thresh_sigma=sigma)
    if mode != "one":
        kw["max_per_beam"] = k
    od, cd = spx.fft_peaks(xd, nfft, spx.WINDOW_HANN, m, **kw)
    xh = xd.cpu()
    if pinned:
        xh = xh.pin_memory()
    else:
        xh = xh.numpy()
    oh, ch = spx.fft_peaks_host(xh, nfft, spx.WINDOW_HANN, m, **kw)
    # page-locked outputs as well: the kernel writes the peaks in place (also
    # behind chunked uploads of pageable input)
    oh2 = torch.zeros(oh.shape, dtype=oh.dtype).pin_memory()
    ch2 = torch.zeros(ch.shape, dtype=ch.dtype).pin_memory()
    spx.fft_peaks_host(xh, nfft, spx.WINDOW_HANN, m, out=oh2, counts=ch2, **kw)
    np.testing.assert_array_equal(ch2.numpy(), ch.numpy())
    g1, g2 = spx.maxvalues_to_numpy(oh), spx.maxvalues_to_numpy(oh2)
    for b in range(beams):
        n = int(ch[b]) if mode != "one" else g1.shape[1]
        np.testing.assert_array_equal(g2[b, :n], g1[b, :n])
    gd, gh = spx.maxvalues_to_numpy(od), spx.maxvalues_to_numpy(oh)
    if mode == "one":
        np.testing.assert_array_equal(gh, gd)
        return
    cd = cd.cpu().numpy()
    np.testing.assert_array_equal(ch.numpy(), cd)
    for b in range(beams):
        np.testing.assert_array_equal(gh[b, : cd[b]], gd[b, : cd[b]])


def _tie_inputs(n):
    """Inputs whose spectra are full of exact magnitude ties and plateaus."""
    rng = np.random.default_rng(n)
    imp = np.zeros((1, n), np.complex64)
    imp[0, 0] = 1.0                       # flat |X| = 1 everywhere
    two = np.zeros((1, n), np.complex64)
    two[0, 0], two[0, 3] = 1.0, 1.0       # |1 + e^{-i 2 pi 3k/N}|: repeating exact values
    dc = np.ones((1, n), np.complex64)    # one line at k = 0
    ints = (rng.integers(-2, 3, (3, n)) + 1j * rng.integers(-2, 3, (3, n))).astype(np.complex64)
    return np.concatenate([imp, two, dc, ints])


@pytest.mark.parametrize("nfft", [4096, 65536, 131072])
@pytest.mark.parametrize("sigma", [0.0, 6.0])
def test_fused_exact_ties(spx, cuda, nfft, sigma):
    """Magnitude comparisons and the noise histogram take the exact square
    root whenever two |X|^2 are too close to decide from |X|^2 alone: spectra
    with exact ties and plateaus give the oracle's lists bit for bit."""
    import torch
    if nfft > 16384 and sigma == 0.0:
        pytest.skip("unthresholded all-maxima with C > 1 runs the composed path")
    x = _tie_inputs(min(nfft, 65536))
    xd = torch.from_numpy(x).to(cuda)
    spec = spx.fft(xd, nfft).cpu().numpy()
    out, counts = spx.fft_peaks(xd, nfft, spx.WINDOW_NONE, spx.PEAK_ALL, sample_rate=1.0,
                                refine=1, thresh_sigma=sigma)
    ref, rc = orc.all_maxima(None, spec, nfft, 1.0, refine=1, thresh_sigma=sigma)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rc)
    assert_rows_equal(spx.maxvalues_to_numpy(out), ref, rc)
    if nfft <= 16384:
        out, counts = spx.fft_peaks(xd, nfft, spx.WINDOW_NONE, spx.PEAK_TOPK, sample_rate=1.0,
                                    max_per_beam=8, refine=1, thresh_sigma=sigma)
        ref, rc = orc.topk(None, spec, nfft, 1.0, 8, thresh_sigma=sigma)
        np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), rc)
        assert_rows_equal(spx.maxvalues_to_numpy(out), ref, rc)


def test_concurrent_large_searches_on_two_streams(spx, cuda):
    """Two contexts on two streams run the large search (cooperative beam-group
    FFT + maxima kernel) at the same time, repeatedly: every result equals the
    serial result and no bounded wait gives up (spx_synchronize is SPX_OK)."""
    import torch
    from spectrum_gb300 import Context
    x = torch.from_numpy(_beams(96, 65536, 17)).to(cuda)
    y = torch.from_numpy(_beams(96, 65536, 18)).to(cuda)
    kw = dict(sample_rate=1.0, refine=1, thresh_sigma=6.0)
    ref_x = [t.clone() for t in spx.fft_peaks(x, 131072, spx.WINDOW_HANN, spx.PEAK_ALL, **kw)]
    ref_y = [t.clone() for t in spx.fft_peaks(y, 131072, spx.WINDOW_HANN, spx.PEAK_ALL, **kw)]
    torch.cuda.synchronize()
    ca, cb = Context(0), Context(0)
    sa, sb = torch.cuda.Stream(), torch.cuda.Stream()
    results = []
    for _ in range(8):
        with torch.cuda.stream(sa):
            ra = spx.fft_peaks(x, 131072, spx.WINDOW_HANN, spx.PEAK_ALL, ctx=ca, **kw)
        with torch.cuda.stream(sb):
            rb = spx.fft_peaks(y, 131072, spx.WINDOW_HANN, spx.PEAK_ALL, ctx=cb, **kw)
        results.append((ra, rb))
    torch.cuda.synchronize()
    for c, s in ((ca, sa), (cb, sb)):
        c.bind_stream(s)
        assert spx.lib.spx_synchronize(c.h) == 0
    for ra, rb in results:
        for got, ref in ((ra, ref_x), (rb, ref_y)):
            assert torch.equal(got[1], ref[1])
            g0, r0, cnt = got[0].cpu(), ref[0].cpu(), ref[1].cpu()
            for b in range(cnt.shape[0]):
                n = min(int(cnt[b]), r0.shape[1])  # rows past a beam's count are not written
                assert torch.equal(g0[b, :n], r0[b, :n])
    ca.close()
    cb.close()
