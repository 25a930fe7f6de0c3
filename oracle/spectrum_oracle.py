"""CPU oracle for the FFT -> |X| -> peaks path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU legs of ``bench.py`` may import this module, and only as the checker or as
the timed CPU baseline; the product path (``spectrum_gb300``) never calls it.

It restates, in numpy, the reference DspSpectrum algorithms for this path:

* window + zero padding: ``pad_data_windowed``
  (include/spectrum/kernels/fft_processor_kernels_rocm.hpp:84-115), window
  values evaluated in FP64 and rounded to FP32 (the reference uses ``__cosf``);
* FFT: pocketfft through ``numpy.fft`` (FP32 input stays FP32 in numpy >= 2),
  the same library the reference vendors for ``CpuFFT::ForwardC2C``
  (include/spectrum/utils/cpu_fft.hpp:68-89); FP64 via complex128;
* magnitude: ``sqrt(re*re + im*im)`` with every FP32 operation rounded
  (complex_to_magnitude, fft_processor_kernels_rocm.hpp:142-154);
* ONE_PEAK / TWO_PEAKS: post_kernel_one_peak / post_kernel_two_peaks
  (include/spectrum/kernels/fft_kernel_sources_rocm.hpp:122-519) including
  the 256-thread tie order of their reductions;
* ALL_MAXIMA: detect_all_maxima + scan + compact_maxima
  (include/spectrum/kernels/all_maxima_kernel_sources_rocm.hpp:57-264) with the
  window defaults of spectrum_processor_rocm.cpp:703-705 and the capacity rule of
  all_maxima_pipeline_rocm.cpp:304-307;
* extensions without a reference counterpart, defined here and in the CUDA
  kernels identically: parabolic refinement of every maximum, top-K of the
  strict local maxima, and the histogram-median noise threshold.
"""
from __future__ import annotations

import math

import numpy as np

MAXVALUE_DTYPE = np.dtype(
    [
        ("index", "<u4"),
        ("real", "<f4"),
        ("imag", "<f4"),
        ("magnitude", "<f4"),
        ("phase", "<f4"),
        ("freq_offset", "<f4"),
        ("refined_frequency", "<f4"),
        ("pad", "<u4"),
    ]
)
assert MAXVALUE_DTYPE.itemsize == 32

RAD_TO_DEG = np.float32(57.29577951)  # fft_kernel_sources_rocm.hpp:247

WINDOW_NONE, WINDOW_HANN, WINDOW_HAMMING, WINDOW_BLACKMAN, WINDOW_BLACKMAN_HARRIS = range(5)
REFINE_NONE, REFINE_PARABOLIC = 0, 1

f32 = np.float32


# ---------------------------------------------------------------------------
# sizes
# ---------------------------------------------------------------------------
def next_pow2(n: int) -> int:
    """fft_processor_rocm.cpp:665-671 (0 -> 1)."""
    if n == 0:
        return 1
    return 1 << (int(n) - 1).bit_length()


def next_smooth23(n: int) -> int:
    """Smallest 2^a 3^b >= n."""
    if n <= 1:
        return 1
    best = None
    p2 = 1
    while p2 < 2 * n:
        v = p2
        while v < n:
            v *= 3
        best = v if best is None else min(best, v)
        p2 *= 2
    return best


def resolve_window(nfft: int, start: int, end: int) -> tuple[int, int]:
    """Search-window defaults of spectrum_processor_rocm.cpp:703-705."""
    if start == 0:
        start = 1
    if end == 0:
        end = nfft // 2
    if end >= nfft:
        end = nfft - 1
    return start, end


def all_maxima_capacity(nfft: int, start: int, end: int, max_per_beam: int) -> tuple[int, int, int]:
    """(start, end, cap) with the unsigned arithmetic of all_maxima_pipeline_rocm.cpp:304-307."""
    start, end = resolve_window(nfft, start, end)
    half = ((end - start) & 0xFFFFFFFF) // 2
    return start, end, min(half, max_per_beam)


def noise_threshold_factor(sigma: float) -> np.float32:
    """(sqrt(pi/2) + s sqrt(2 - pi/2)) / sqrt(2 ln 2), rounded to FP32."""
    return f32((math.sqrt(math.pi / 2) + sigma * math.sqrt(2 - math.pi / 2)) / math.sqrt(2 * math.log(2)))


# ---------------------------------------------------------------------------
# window, FFT, magnitude
# ---------------------------------------------------------------------------
def window(kind: int, n_point: int) -> np.ndarray | None:
    """FP32 window with the reference's (n_point - 1) denominator; None for rectangular."""
    if kind == WINDOW_NONE:
        return None
    if n_point < 2:
        return np.ones(n_point, np.float32)
    th = 2.0 * np.pi * np.arange(n_point, dtype=np.float64) / (n_point - 1)
    if kind == WINDOW_HANN:
        w = 0.5 * (1.0 - np.cos(th))
    elif kind == WINDOW_HAMMING:
        w = 0.54 - 0.46 * np.cos(th)
    elif kind == WINDOW_BLACKMAN:
        w = 0.42 - 0.5 * np.cos(th) + 0.08 * np.cos(2 * th)
    elif kind == WINDOW_BLACKMAN_HARRIS:
        w = 0.35875 - 0.48829 * np.cos(th) + 0.14128 * np.cos(2 * th) - 0.01168 * np.cos(3 * th)
    else:
        raise ValueError(f"unknown window {kind}")
    return w.astype(np.float32)


def windowed(x: np.ndarray, kind: int) -> np.ndarray:
    """x [beams, n_point] complex64 times the FP32 window (each product rounded)."""
    w = window(kind, x.shape[-1])
    if w is None:
        return x.astype(np.complex64, copy=False)
    re = x.real.astype(np.float32) * w
    im = x.imag.astype(np.float32) * w
    return (re + 1j * im).astype(np.complex64)


def fft_fp32(x: np.ndarray, nfft: int, win: int = WINDOW_NONE) -> np.ndarray:
    """Windowed, zero-padded forward FFT in FP32 (pocketfft via numpy)."""
    xw = windowed(np.atleast_2d(x), win)
    out = np.fft.fft(xw, n=nfft, axis=-1)
    assert out.dtype == np.complex64, "numpy >= 2 keeps FP32 FFTs in FP32"
    return out


def ifft_fp32(X: np.ndarray) -> np.ndarray:
    """Inverse C2C with 1/N in FP32 (pocketfft via numpy): CpuFFT::InverseC2C
    (include/spectrum/utils/cpu_fft.hpp:96-118, backward c2c with fct 1/N)."""
    out = np.fft.ifft(np.atleast_2d(X).astype(np.complex64), axis=-1)
    assert out.dtype == np.complex64
    return out


def fft_r2c_fp32(x: np.ndarray, nfft: int, win: int = WINDOW_NONE, full: bool = False) -> np.ndarray:
    """Real-input FFT in FP32: CpuFFT::ForwardR2C (nfft/2 + 1 bins,
    cpu_fft.hpp:131-152) or ForwardR2C_Full (nfft bins, upper half
    conj(X[nfft - k]), cpu_fft.hpp:165-180), after window and zero padding."""
    xr = np.atleast_2d(x).astype(np.float32)
    w = window(win, xr.shape[-1])
    if w is not None:
        xr = (xr * w).astype(np.float32)
    half = np.fft.rfft(xr, n=nfft, axis=-1).astype(np.complex64)
    if not full:
        return half
    out = np.empty(xr.shape[:-1] + (nfft,), np.complex64)
    out[..., : half.shape[-1]] = half
    k = np.arange(half.shape[-1], nfft)
    out[..., k] = np.conj(half[..., nfft - k])
    return out


def fft_fp64(x: np.ndarray, nfft: int, win: int = WINDOW_NONE) -> np.ndarray:
    """The same transform in FP64 (window in FP64 too): the accuracy reference."""
    x = np.atleast_2d(x).astype(np.complex128)
    if win != WINDOW_NONE:
        n = x.shape[-1]
        th = 2.0 * np.pi * np.arange(n) / max(n - 1, 1)
        w = {
            WINDOW_HANN: lambda: 0.5 * (1.0 - np.cos(th)),
            WINDOW_HAMMING: lambda: 0.54 - 0.46 * np.cos(th),
            WINDOW_BLACKMAN: lambda: 0.42 - 0.5 * np.cos(th) + 0.08 * np.cos(2 * th),
            WINDOW_BLACKMAN_HARRIS: lambda: 0.35875 - 0.48829 * np.cos(th)
            + 0.14128 * np.cos(2 * th) - 0.01168 * np.cos(3 * th),
        }[win]()
        if n < 2:
            w = np.ones(n)
        x = x * w
    return np.fft.fft(x, n=nfft, axis=-1)


def mag2_rn(z: np.ndarray) -> np.ndarray:
    re = z.real.astype(np.float32)
    im = z.imag.astype(np.float32)
    return re * re + im * im  # two rounded products, one rounded sum


def mag_rn(z: np.ndarray) -> np.ndarray:
    return np.sqrt(mag2_rn(z))


def magnitude(z: np.ndarray, inv_n: float = 1.0, squared: bool = False) -> np.ndarray:
    """complex_to_magnitude(_squared): |z| * inv_n (or |z|^2 * inv_n)."""
    m = mag2_rn(z) if squared else mag_rn(z)
    return m * f32(inv_n)


def mag_phase(z: np.ndarray) -> np.ndarray:
    """complex_to_mag_phase: interleaved {|z|, atan2(im, re)} as float32 [..., 2]."""
    out = np.empty(z.shape + (2,), np.float32)
    out[..., 0] = mag_rn(z)
    out[..., 1] = np.arctan2(z.imag.astype(np.float32), z.real.astype(np.float32))
    return out


def inv_n_from_norm(norm_coeff: float, n_point: int) -> float:
    """ComplexToMagPhaseROCm::ComputeInvN (complex_to_mag_phase_rocm.cpp:170-176)."""
    if norm_coeff < 0:
        return float(f32(1.0) / f32(n_point)) if n_point > 0 else 1.0
    if norm_coeff > 0:
        return float(norm_coeff)
    return 1.0


# ---------------------------------------------------------------------------
# peak helpers
# ---------------------------------------------------------------------------
def _phase_deg(re, im) -> np.float32:
    return f32(np.arctan2(f32(im), f32(re))) * RAD_TO_DEG


def parabolic(yl, yc, yr) -> tuple[bool, np.float32]:
    """fft_kernel_sources_rocm.hpp:229-239: clamped 3-point offset, 0 if |den| <= 1e-10."""
    yl, yc, yr = f32(yl), f32(yc), f32(yr)
    denom = (yl - f32(2.0) * yc) + yr
    if abs(denom) > f32(1e-10):
        fo = (f32(0.5) * (yl - yr)) / denom
        fo = min(max(fo, f32(-0.5)), f32(0.5))
        return True, f32(fo)
    return False, f32(0.0)


def _bin_width(fs: float, nfft: int) -> np.float32:
    return f32(fs) / f32(nfft)


def _write_peak4(f: np.ndarray, nfft: int, ci: int, fs: float, mirror: bool) -> np.ndarray:
    """The 4 MaxValue of post_kernel_one_peak (fft_kernel_sources_rocm.hpp:212-286)."""
    out = np.zeros(4, MAXVALUE_DTYPE)
    fs32 = f32(fs)
    bw = _bin_width(fs, nfft)
    cv = f[ci]
    yc = mag_rn(np.array([cv]))[0]
    hl, hr = ci > 0, ci < nfft - 1
    lv = f[ci - 1] if hl else np.complex64(0)
    rv = f[ci + 1] if hr else np.complex64(0)
    yl = mag_rn(np.array([lv]))[0] if hl else f32(0)
    yr = mag_rn(np.array([rv]))[0] if hr else f32(0)
    fo = f32(0)
    rf = f32(ci) * bw
    if hl and hr:
        ok, fo = parabolic(yl, yc, yr)
        if ok:
            rf = (f32(ci) + fo) * bw
    if mirror:
        rf = fs32 - rf
    pc = _phase_deg(cv.real, cv.imag)
    out[0] = (ci, cv.real, cv.imag, yc, pc, fo, rf, 0)
    rfl = f32(ci - 1) * bw if hl else f32(0)
    if mirror and hl:
        rfl = fs32 - rfl
    out[1] = (ci - 1 if hl else 0, lv.real, lv.imag, yl, _phase_deg(lv.real, lv.imag) if hl else 0, 0, rfl, 0)
    rfc = f32(ci) * bw
    if mirror:
        rfc = fs32 - rfc
    out[2] = (ci, cv.real, cv.imag, yc, pc, 0, rfc, 0)
    rfr = f32(ci + 1) * bw if hr else f32(0)
    if mirror and hr:
        rfr = fs32 - rfr
    out[3] = (ci + 1 if hr else 0, rv.real, rv.imag, yr, _phase_deg(rv.real, rv.imag) if hr else 0, 0, rfr, 0)
    return out


_BITREV8 = np.array([int(f"{i:08b}"[::-1], 2) for i in range(256)], np.int64)


def _argmax_ref_order(vals: np.ndarray) -> int | None:
    """Argmax with the reference reduction's tie order.

    post_kernel_one_peak scans a range with 256 threads (thread lid visits
    offsets lid, lid+256, ... keeping its FIRST strict maximum), then reduces
    local[lid] with local[lid+stride] for stride = 128, 64, ..., 1, keeping
    local[lid] on ties (fft_kernel_sources_rocm.hpp:151-192).  The last merge
    (stride 1) prefers even lids, the one before prefers lid bit 1 = 0, and so
    on: among equal maxima the winner has the smallest bit-reversed lid
    (8 bits), then the smallest offset.  Returns the offset, or None when no
    value is a number."""
    ok = ~np.isnan(vals)
    if not ok.any():
        return None
    m = np.max(vals[ok])
    t = np.nonzero(vals == m)[0]
    key = _BITREV8[t % 256] * (1 << 24) + (t // 256)
    return int(t[np.argmin(key)])


def one_two_peaks(fft: np.ndarray, nfft: int, search_range: int, fs: float, two: bool) -> np.ndarray:
    """ONE_PEAK -> [beams, 4] MaxValue, TWO_PEAKS -> [beams, 8]."""
    fft = np.asarray(fft, np.complex64).reshape(-1, nfft)
    if search_range == 0:
        search_range = nfft // 4
    half = search_range // 2
    r0 = nfft - half
    mags = mag_rn(fft)
    out = np.zeros((fft.shape[0], 8 if two else 4), MAXVALUE_DTYPE)
    for b in range(fft.shape[0]):
        tl = _argmax_ref_order(mags[b, :half])
        tr = _argmax_ref_order(mags[b, r0:])
        il, ml = (tl, mags[b, tl]) if tl is not None else (0, f32(-1.0))
        ir, mr = (r0 + tr, mags[b, r0 + tr]) if tr is not None else (r0, f32(-1.0))
        if two:
            out[b, :4] = _write_peak4(fft[b], nfft, il, fs, False)
            out[b, 4:] = _write_peak4(fft[b], nfft, ir, fs, True)
        else:
            right = mr > ml
            out[b] = _write_peak4(fft[b], nfft, ir if right else il, fs, right)
    return out


def _make_max(fft_row, mag_row, k: int, bw, refine: int):
    z = fft_row[k]
    yc = mag_row[k]
    fo = f32(0)
    rf = f32(k) * bw
    if refine == REFINE_PARABOLIC:
        ok, fo = parabolic(mag_row[k - 1], yc, mag_row[k + 1])
        if ok:
            rf = (f32(k) + fo) * bw
    return (k, z.real, z.imag, yc, _phase_deg(z.real, z.imag), fo, rf, 0)


def local_maxima(mag_row: np.ndarray, start: int, end: int, thr=None) -> np.ndarray:
    """Strict local maxima in [start, end) (detect_all_maxima), above thr if given."""
    if end <= start:
        return np.zeros(0, np.int64)
    i = np.arange(start, end)
    c = mag_row[i]
    f = (c > mag_row[i - 1]) & (c > mag_row[i + 1])
    if thr is not None:
        f &= c > thr
    return i[f]


def noise_threshold(mag: np.ndarray, start: int, end: int, factor) -> np.ndarray:
    """Per-beam threshold = histogram-interpolated median of |X| over [start, end) * factor.

    bucket = (bits & 0x7fffffff) >> 19; r = (n-1)//2; bucket b holds rank r;
    frac = (float(r - below) + 0.5) / float(h[b]); med = lo + (hi - lo) * frac
    (FP32, each step rounded); thr = med * factor.  n == 0 -> +inf."""
    mag = np.asarray(mag, np.float32)
    beams = mag.shape[0]
    n = max(end - start, 0)
    thr = np.full(beams, np.inf, np.float32)
    if n == 0:
        return thr
    r = (n - 1) // 2
    for b in range(beams):
        bits = mag[b, start:end].view(np.uint32) & np.uint32(0x7FFFFFFF)
        h = np.bincount(bits >> np.uint32(19), minlength=4096)
        cum = np.cumsum(h)
        bk = int(np.searchsorted(cum, r, side="right"))
        below = int(cum[bk] - h[bk])
        lo = np.array([bk << 19], np.uint32).view(np.float32)[0]
        hi = np.array([(bk + 1) << 19], np.uint32).view(np.float32)[0]
        frac = (f32(r - below) + f32(0.5)) / f32(h[bk])
        med = lo + (hi - lo) * frac
        thr[b] = med * f32(factor)
    return thr


def all_maxima(mag, fft, nfft: int, fs: float, search_start: int = 0, search_end: int = 0,
               max_per_beam: int = 1000, refine: int = REFINE_NONE, thresh_sigma: float = 0.0):
    """IAllMaximaPipeline::Execute semantics -> (maxima [beams, cap], counts [beams]).

    counts are the untruncated numbers of maxima (compact_maxima writes
    scan[n-1] + flag[n-1]); rows hold min(count, cap) valid entries."""
    fft = np.asarray(fft, np.complex64).reshape(-1, nfft)
    mag = mag_rn(fft) if mag is None else np.asarray(mag, np.float32).reshape(-1, nfft)
    start, end, cap = all_maxima_capacity(nfft, search_start, search_end, max_per_beam)
    beams = fft.shape[0]
    thr = None
    if thresh_sigma > 0:
        thr = noise_threshold(mag, start, end, noise_threshold_factor(thresh_sigma))
    out = np.zeros((beams, cap), MAXVALUE_DTYPE)
    counts = np.zeros(beams, np.uint32)
    bw = _bin_width(fs, nfft)
    for b in range(beams):
        pos = local_maxima(mag[b], start, end, None if thr is None else thr[b])
        counts[b] = len(pos)
        for r, k in enumerate(pos[:cap]):
            out[b, r] = _make_max(fft[b], mag[b], int(k), bw, refine)
    return out, counts


def topk(mag, fft, nfft: int, fs: float, k: int, search_start: int = 0, search_end: int = 0,
         refine: int = REFINE_PARABOLIC, thresh_sigma: float = 0.0):
    """K largest strict local maxima in [start, end): |X| descending, ties by lower bin.
    -> (maxima [beams, K], counts [beams] = entries written)."""
    fft = np.asarray(fft, np.complex64).reshape(-1, nfft)
    mag = mag_rn(fft) if mag is None else np.asarray(mag, np.float32).reshape(-1, nfft)
    start, end = resolve_window(nfft, search_start, search_end)
    beams = fft.shape[0]
    thr = None
    if thresh_sigma > 0:
        thr = noise_threshold(mag, start, end, noise_threshold_factor(thresh_sigma))
    out = np.zeros((beams, k), MAXVALUE_DTYPE)
    counts = np.zeros(beams, np.uint32)
    bw = _bin_width(fs, nfft)
    for b in range(beams):
        pos = local_maxima(mag[b], start, end, None if thr is None else thr[b])
        order = np.lexsort((pos, -mag[b, pos]))[:k]
        counts[b] = len(order)
        for r, i in enumerate(pos[order]):
            out[b, r] = _make_max(fft[b], mag[b], int(i), bw, refine)
    return out, counts


def fft_peaks(x: np.ndarray, nfft: int, win: int, mode: str, fs: float, **kw):
    """Composed path: window + pad + FFT (FP32) + |X| + peak search."""
    spec = fft_fp32(x, nfft, win)
    if mode == "one":
        return one_two_peaks(spec, nfft, kw.get("search_range", 0), fs, False), None
    if mode == "two":
        return one_two_peaks(spec, nfft, kw.get("search_range", 0), fs, True), None
    if mode == "all":
        return all_maxima(None, spec, nfft, fs, kw.get("search_start", 0), kw.get("search_end", 0),
                          kw.get("max_per_beam", 1000), kw.get("refine", REFINE_NONE),
                          kw.get("thresh_sigma", 0.0))
    return topk(None, spec, nfft, fs, kw.get("k", 5), kw.get("search_start", 0), kw.get("search_end", 0),
                kw.get("refine", REFINE_PARABOLIC), kw.get("thresh_sigma", 0.0))
