"""GPU parity of the batched FFT (window + zero padding + epilogues) and of the
magnitude kernels against the oracle (numpy pocketfft FP32 / FP64).

Tolerances: spectra within 1e-5 of the beam's largest |X| (FP32 reference and
FP64 reference alike); |X| and |X|^2 outputs bit-exact against the same
formula applied to the kernel's own complex output; phase within 4e-6 rad.
"""
import numpy as np
import pytest

from oracle import spectrum_oracle as orc

pytestmark = pytest.mark.gpu

FFT_TOL = 1e-5

# (nfft, n_point, window): every cluster size (1, 2, 3, 4, 6, 8, 9, 16 CTAs per
# beam), every radix, zero padding and the four windows.
FFT_CASES = [
    (2, 2, 0), (3, 3, 0), (4, 3, 0), (6, 5, 1), (8, 8, 0), (9, 9, 2), (12, 7, 0), (16, 10, 3),
    (64, 64, 0), (243, 200, 1), (1024, 1000, 1), (1152, 1152, 0), (2187, 2000, 4),
    (4096, 4096, 1), (6561, 6561, 0), (13122, 13000, 2), (13824, 13824, 0), (16384, 16384, 1),
    (17496, 17000, 0), (19683, 19683, 0), (32768, 20000, 1), (52488, 52000, 0),
    (65536, 65536, 3), (69984, 69000, 1), (104976, 100000, 1), (131072, 65536, 1),
    (59049, 59049, 0), (262144, 262144, 0), (1 << 19, 300000, 1), (1 << 20, 1 << 20, 4),
    (1 << 21, 1 << 20, 1),  # nextPow2(2^20) x repeat_count 2, the reference's largest common FFTProcessor size
    (1 << 22, 1 << 20, 1),  # nextPow2(2^20) x repeat_count 4: the four-step transform (2048 x 2048)
    (3 << 21, 5000000, 4),  # 3-smooth above 2^21 (1536 x 4096), Blackman-Harris
    (1 << 23, 1 << 23, 0),  # 2048 x 4096, no padding
]


def _signal(beams, n, seed):
    rng = np.random.default_rng(seed)
    return ((rng.standard_normal((beams, n)) + 1j * rng.standard_normal((beams, n))) /
            np.sqrt(2)).astype(np.complex64)


def _max_rel(a, b):
    scale = np.abs(b).max(axis=-1, keepdims=True)
    return float((np.abs(a - b) / scale).max())


@pytest.mark.parametrize("nfft,n_point,win", FFT_CASES)
def test_fft_complex_matches_pocketfft(spx, cuda, nfft, n_point, win):
    import torch
    beams = 3 if nfft <= 65536 else (2 if nfft <= 262144 or nfft >= (1 << 22) else 1)
    x = _signal(beams, n_point, nfft + n_point)
    got = spx.fft(torch.from_numpy(x).to(cuda), nfft, window=win).cpu().numpy()
    ref32 = orc.fft_fp32(x, nfft, win)
    ref64 = orc.fft_fp64(x, nfft, win)
    e32 = _max_rel(got, ref32)
    e64 = _max_rel(got, ref64)
    assert e32 < FFT_TOL, f"vs FP32 pocketfft: {e32:.3e}"
    assert e64 < FFT_TOL, f"vs FP64 pocketfft: {e64:.3e}"


def test_pipelined_column_tiles_match_single_tiles_and_pocketfft(spx, cuda):
    """2^19 points run the pipelined column kernel: with 8 beams (1024 column
    tiles) every CTA loops over several tiles, streaming the next one into
    shared memory while it transforms the current one and alternating its two
    exchange tiles.  Each beam equals the same beam transformed alone (128
    tiles: one per CTA) bit for bit, and pocketfft within the tolerance."""
    import torch
    nfft, n_point = 1 << 19, 400000
    x = _signal(8, n_point, 77)
    xd = torch.from_numpy(x).to(cuda)
    got = spx.fft(xd, nfft, window=spx.WINDOW_HANN).cpu().numpy()
    for b in (0, 3, 7):
        alone = spx.fft(xd[b:b + 1].contiguous(), nfft, window=spx.WINDOW_HANN).cpu().numpy()
        assert np.array_equal(got[b:b + 1].view(np.uint32), alone.view(np.uint32)), f"beam {b}"
    for b in (0, 7):
        e32 = _max_rel(got[b:b + 1], orc.fft_fp32(x[b:b + 1], nfft, orc.WINDOW_HANN))
        assert e32 < FFT_TOL, f"beam {b} vs FP32 pocketfft: {e32:.3e}"


@pytest.mark.parametrize("nfft,n_point", [(4096, 4000), (131072, 65536), (13122, 13122), (1 << 19, 400000),
                                          (1 << 20, 1 << 20), (1 << 21, 1500000)])
def test_fft_epilogues_consistent(spx, cuda, nfft, n_point):
    """MAG / MAG2 / MAGPHASE come from the same transform as COMPLEX."""
    import torch
    x = torch.from_numpy(_signal(2, n_point, 7)).to(cuda)
    z = spx.fft(x, nfft, window=spx.WINDOW_HANN).cpu().numpy()
    m = spx.fft(x, nfft, window=spx.WINDOW_HANN, out="mag", scale=0.25).cpu().numpy()
    m2 = spx.fft(x, nfft, window=spx.WINDOW_HANN, out="mag2", scale=0.5).cpu().numpy()
    mp = spx.fft(x, nfft, window=spx.WINDOW_HANN, out="magphase").cpu().numpy()
    np.testing.assert_array_equal(m, orc.magnitude(z, 0.25))
    np.testing.assert_array_equal(m2, orc.magnitude(z, 0.5, squared=True))
    np.testing.assert_array_equal(mp[..., 0], orc.mag_rn(z))
    np.testing.assert_allclose(mp[..., 1], np.arctan2(z.imag, z.real), rtol=0, atol=4e-6)


@pytest.mark.parametrize("count,offset", [(1, 0), (7, 0), (1 << 20, 0), (1001, 1), (12345, 0)])
@pytest.mark.parametrize("squared", [False, True])
def test_magnitude_kernel_bit_exact(spx, cuda, count, offset, squared):
    """ComplexToMagPhase::ProcessMagnitude semantics, including odd counts and
    an input not aligned to 16 bytes (scalar path)."""
    import torch
    z = _signal(1, count + offset, count)[0]
    zt = torch.from_numpy(z).to(cuda)[offset:]
    inv_n = orc.inv_n_from_norm(-1.0, count)
    got = spx.magnitude(zt, inv_n=inv_n, squared=squared).cpu().numpy()
    np.testing.assert_array_equal(got, orc.magnitude(z[offset:], inv_n, squared))


def test_magnitude_known_values(spx, cuda):
    """3-4-5 triangle, zero, tiny values (tests/test_complex_to_mag_phase_rocm.hpp:239-259)."""
    import torch
    z = np.array([3 + 4j, 0, 1e-6 + 1e-6j, -3 - 4j], np.complex64)
    got = spx.magnitude(torch.from_numpy(z).to(cuda)).cpu().numpy()
    np.testing.assert_array_equal(got[[0, 1, 3]], np.float32([5, 0, 5]))
    assert abs(got[2] - np.float32(np.sqrt(2e-12))) < 1e-12
    mp = spx.mag_phase(torch.from_numpy(z).to(cuda)).cpu().numpy()
    np.testing.assert_allclose(mp[:, 1], np.arctan2(z.imag, z.real), atol=4e-6)


def test_fft_rejects_bad_sizes(spx, cuda):
    import torch
    x = torch.zeros((1, 100), dtype=torch.complex64, device=cuda)
    with pytest.raises(ValueError):
        spx.fft(x, 50)           # nfft < n_point
    with pytest.raises(ValueError):
        spx.fft(x, (1 << 27) + 1)  # no direct plan, too long for Bluestein's transform
    with pytest.raises(ValueError):
        spx.fft(x, 1 << 29)        # beyond the four-step transform's 2^28
    with pytest.raises(ValueError):
        spx.fft(x, 3 ** 18)        # 3-smooth beyond 2^28


def test_precision_workload_dynamic_range(spx, cuda):
    """Two tones 120 dB apart + noise 1e-7, Blackman-Harris, 2^20 points: the
    FP32 transform (FP64-generated twiddles) stays within 1e-6 of the FP64
    spectrum's peak and the weak tone stands far above the error floor."""
    import torch
    from spectrum_gb300 import synth
    bs = synth.workload_precision(seed=3, beams=8)
    x = synth.synth_numpy(bs)
    n = 1 << 20
    got = spx.fft(torch.from_numpy(x).to(cuda), n, window=spx.WINDOW_BLACKMAN_HARRIS).cpu().numpy()
    ref = orc.fft_fp64(x, n, orc.WINDOW_BLACKMAN_HARRIS)
    for b in range(8):
        peak = np.abs(ref[b]).max()
        err = np.abs(got[b] - ref[b])
        assert err.max() / peak < 1e-6, err.max() / peak
        rms = np.sqrt(np.mean(err ** 2))
        weak = int(round(bs.freqs[b][1] * n))
        weak_mag = np.abs(got[b, weak - 2:weak + 3]).max()
        assert 20 * np.log10(peak / rms) > 150          # dynamic range vs the FP32 error floor
        assert 20 * np.log10(weak_mag / rms) > 40       # the -120 dB tone is visible


BIN_REL_TOL = 1e-5


@pytest.mark.parametrize("workload", ["small", "large", "uneven", "precision", "learned"])
def test_magnitude_per_bin_relative_error(spx, cuda, workload):
    """|X| per bin within 1e-5 relative of pocketfft's FP32 |X| and of the
    FP64 |X|, on every bin 20 dB or more above the beam's median |X| (the
    noise floor) and within 60 dB of its peak, for beams of each benchmark
    workload.  (The whole-spectrum bound above is 1e-5 of the beam's peak.)"""
    import torch
    from spectrum_gb300 import synth
    win = spx.WINDOW_BLACKMAN_HARRIS if workload == "precision" else spx.WINDOW_HANN
    if workload == "small":
        bs, rows = synth.workload_small(seed=0), range(8)
    elif workload == "large":
        bs, rows = synth.workload_large(seed=1, beams=4), range(4)
    elif workload == "uneven":
        bs, rows = synth.workload_uneven(seed=2, beams=64), range(0, 64, 8)
    elif workload == "precision":
        bs, rows = synth.workload_precision(seed=3, beams=2), range(2)
    else:
        bs, rows = synth.workload_learned(seed=4, beams=8), range(8)
    xs = synth.synth_numpy(bs)
    checked = 0
    for b in rows:
        n = int(bs.lengths[b])
        x = np.ascontiguousarray(xs[b:b + 1, :n])
        nfft = {"small": 4096, "large": 131072, "precision": 1 << 20, "learned": 8192}.get(
            workload, orc.next_smooth23(n))
        got = np.abs(spx.fft(torch.from_numpy(x).to(cuda), nfft, window=win).cpu().numpy()[0]).astype(np.float64)
        a64 = np.abs(orc.fft_fp64(x, nfft, win)[0])
        a32 = np.abs(orc.fft_fp32(x, nfft, win)[0]).astype(np.float64)
        sel = (a64 >= 10.0 * np.median(a64)) & (a64 >= 1e-3 * a64.max())
        assert sel.sum() > 0
        r64 = float((np.abs(got[sel] - a64[sel]) / a64[sel]).max())
        r32 = float((np.abs(got[sel] - a32[sel]) / a32[sel]).max())
        assert r64 < BIN_REL_TOL, f"beam {b}: {r64:.3e} vs FP64"
        assert r32 < BIN_REL_TOL, f"beam {b}: {r32:.3e} vs FP32 pocketfft"
        checked += int(sel.sum())
    assert checked >= 10


# ---- inverse and real-input transforms (CpuFFT::InverseC2C / ForwardR2C / ForwardR2C_Full) ----

def _golden():
    from pathlib import Path
    return np.load(Path(__file__).parent / "golden" / "reference_golden.npz")


@pytest.mark.parametrize("n", [64, 1000, 4096, 4374])
def test_fft_any_length_matches_reference_cpufft(spx, cuda, n):
    """CpuFFT::ForwardC2C takes any length; so does spx_fft up to 2^20 points
    (1000 = 2^3 5^3 by Bluestein's transform, 4374 = 2 3^7 by the Stockham
    plan): the reference's own outputs (golden) within 1e-5 of the peak."""
    import torch
    G = _golden()
    x, X = G[f"fft{n}_x"], G[f"fft{n}_X"]
    got = spx.fft(torch.from_numpy(x).to(cuda), n).cpu().numpy()
    assert np.abs(got - X).max() / np.abs(X).max() < FFT_TOL


@pytest.mark.parametrize("nfft,n_point,win", [(5, 5, 0), (7, 6, 1), (1000, 900, 1), (1009, 1009, 4), (65537, 60000, 1),
                                              ((1 << 20) - 1, 1 << 19, 2), (3 << 18, 700000, 0),
                                              ((1 << 20) + 1, 1 << 20, 1), (5000011, 4000000, 1)])
def test_bluestein_lengths_match_fp64(spx, cuda, nfft, n_point, win):
    """Lengths without a Stockham plan (primes, 5- and 7-smooth, 2^20 - 1,
    3 2^18, 2^20 + 1 and the prime 5000011, whose power-of-two transforms of
    2^22 and 2^24 points run the four-step path): every output mode against
    the FP64 transform of the windowed, zero-padded samples, within 1e-5 of
    the peak; the inverse round-trips."""
    import torch
    beams = 2 if nfft < (1 << 19) else 1
    x = _signal(beams, n_point, nfft)
    xd = torch.from_numpy(x).to(cuda)
    ref = orc.fft_fp64(x, nfft, win)
    got = spx.fft(xd, nfft, window=win).cpu().numpy()
    peak = np.abs(ref).max()
    assert np.abs(got - ref).max() / peak < FFT_TOL
    mag = spx.fft(xd, nfft, window=win, out="mag").cpu().numpy()
    assert np.abs(mag - np.abs(ref)).max() / peak < FFT_TOL
    back = spx.ifft(spx.fft(xd, nfft)).cpu().numpy()
    xp = np.zeros((beams, nfft), np.complex64)
    xp[:, :n_point] = x
    assert np.abs(back - xp).max() / np.abs(xp).max() < 1e-5


@pytest.mark.parametrize("n", [64, 1000, 4096])
def test_ifft_and_r2c_match_reference_cpufft(spx, cuda, n):
    """Against the reference's own CpuFFT outputs (golden): 1e-5 of the peak,
    at 2^a 3^b lengths and at 1000 = 2^3 5^3 (Bluestein's transform)."""
    import torch
    G = _golden()
    X, x = G[f"ifft{n}_X"], G[f"ifft{n}_x"]
    got = spx.ifft(torch.from_numpy(X).to(cuda)).cpu().numpy()
    assert np.abs(got - x).max() / np.abs(x).max() < FFT_TOL
    r, half, full = G[f"r2c{n}_x"], G[f"r2c{n}_half"], G[f"r2c{n}_full"]
    rd = torch.from_numpy(r).to(cuda)
    gh = spx.fft_r2c(rd).cpu().numpy()
    gf = spx.fft_r2c(rd, full=True).cpu().numpy()
    assert gh.shape == half.shape and gf.shape == full.shape
    assert np.abs(gh - half).max() / np.abs(half).max() < FFT_TOL
    assert np.abs(gf - full).max() / np.abs(full).max() < FFT_TOL
    k = np.arange(n // 2 + 1, n)  # the mirror is exact, as in the reference
    np.testing.assert_array_equal(gf[:, k], np.conj(gf[:, n - k]))
    np.testing.assert_array_equal(gf[:, : n // 2 + 1], gh)


@pytest.mark.parametrize("nfft", [2, 9, 96, 4096, 13122, 65536, 131072, 1 << 20, 1 << 21, 1 << 22, 3 << 21])
def test_ifft_round_trip_and_fp64(spx, cuda, nfft):
    import torch
    beams = 2 if nfft < (1 << 20) else 1
    x = _signal(beams, nfft, nfft)
    xd = torch.from_numpy(x).to(cuda)
    back = spx.ifft(spx.fft(xd)).cpu().numpy()
    assert np.abs(back - x).max() / np.abs(x).max() < 3e-6
    got = spx.ifft(xd).cpu().numpy()
    ref = np.fft.ifft(x.astype(np.complex128), axis=-1)
    assert np.abs(got - ref).max() / np.abs(ref).max() < FFT_TOL
    inplace = xd.clone()
    spx.ifft(inplace, out=inplace)
    np.testing.assert_array_equal(inplace.cpu().numpy(), got)


@pytest.mark.parametrize("n_point,nfft,win,full", [(1000, 1024, 1, False), (6000, 6561, 4, True),
                                                   (30000, 32768, 2, False), (2187, 2187, 0, True),
                                                   (1000000, 1 << 20, 1, True), (300000, 1 << 19, 4, False)])
def test_r2c_window_and_padding(spx, cuda, n_point, nfft, win, full):
    import torch
    if not spx.fft_size_supported(nfft):
        pytest.skip("size")
    r = np.random.default_rng(n_point).standard_normal((3, n_point)).astype(np.float32)
    got = spx.fft_r2c(torch.from_numpy(r).to(cuda), nfft, window=win, full=full).cpu().numpy()
    ref = orc.fft_r2c_fp32(r, nfft, win, full)
    assert np.abs(got - ref).max() / np.abs(ref).max() < FFT_TOL


@pytest.mark.parametrize("nfft,n_point", [(1 << 22, 3000000), (1 << 24, 1 << 24)])
def test_four_step_transform_modes_and_peaks(spx, cuda, nfft, n_point):
    """Transforms above 2^21 points (the reference's nextPow2(n_point) x
    repeat_count, fft_processor_rocm.cpp:673-677): |X| and |X|^2 epilogues
    bit-exact against the formula on the complex output, the FP64 spectrum
    within 1e-5 of the peak, and the top-K / all-maxima searches on the same
    spectrum bit-exact against the oracle."""
    import torch
    x = _signal(1, n_point, nfft + 3)
    xd = torch.from_numpy(x).to(cuda)
    z = spx.fft(xd, nfft, window=spx.WINDOW_HANN).cpu().numpy()
    ref = orc.fft_fp64(x, nfft, orc.WINDOW_HANN)
    assert _max_rel(z, ref) < FFT_TOL
    mag = spx.fft(xd, nfft, window=spx.WINDOW_HANN, out="mag").cpu().numpy()
    np.testing.assert_array_equal(mag, orc.magnitude(z))
    out, counts = spx.fft_peaks(xd, nfft, spx.WINDOW_HANN, spx.PEAK_TOPK, sample_rate=1.0, max_per_beam=8,
                                refine=spx.REFINE_PARABOLIC)
    got = spx.maxvalues_to_numpy(out)
    want, wc = orc.topk(None, z, nfft, 1.0, 8)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), wc)
    np.testing.assert_array_equal(got["index"], want["index"])
    np.testing.assert_array_equal(got["refined_frequency"], want["refined_frequency"])
