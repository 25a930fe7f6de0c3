"""spectrum_gb300 — GB300-native FFT -> |X| -> peaks (DspSpectrum's hot path).

The compute path is the native library ``lib/libspectrum_gb300.so`` (CUDA
kernels for sm_103a behind the C ABI of ``include/spx.h``).  This package
binds it with ctypes and offers two layers on top:

* tensor functions (``fft``, ``magnitude``, ``all_maxima`` ...) that take and
  return CUDA ``torch.Tensor`` objects and run on torch's current stream;
* ``spectrum_gb300.dsp_spectrum``: classes mirroring the reference's Python
  module ``dsp_spectrum`` (FFTProcessorROCm, SpectrumMaximaFinderROCm,
  ComplexToMagROCm) for drop-in use; ``batch`` (uneven beams) and
  ``learned`` (learned sub-bin refinement).

PyTorch is used only for device memory and streams.  There is no CPU
fallback: without the native library and a CUDA device every call raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import (OUT_COMPLEX, OUT_MAG, OUT_MAG2, OUT_MAGPHASE, PEAK_ALL, PEAK_ONE, PEAK_TOPK,
                    PEAK_TWO, REFINE_NONE, REFINE_PARABOLIC, WINDOW_BLACKMAN,
                    WINDOW_BLACKMAN_HARRIS, WINDOW_HAMMING, WINDOW_HANN, WINDOW_NONE, SpxError,
                    SpxInvalidArgument, check, lib, peak_params)

MAXVALUE_DTYPE = np.dtype(
    [("index", "<u4"), ("real", "<f4"), ("imag", "<f4"), ("magnitude", "<f4"), ("phase", "<f4"),
     ("freq_offset", "<f4"), ("refined_frequency", "<f4"), ("pad", "<u4")])

_OUT_MODES = {"complex": OUT_COMPLEX, "mag": OUT_MAG, "mag2": OUT_MAG2, "magphase": OUT_MAGPHASE}


def _torch():
    import torch
    return torch


class Context:
    """Owns one ``spx_ctx`` (device + cached plans + scratch).  Each call binds
    the context to torch's current CUDA stream before launching."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib.spx_create(int(device), C.byref(h)))
        self.h = h
        self.device = int(device)

    def close(self) -> None:
        if self.h:
            lib.spx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bind_stream(self, stream=None) -> None:
        torch = _torch()
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        check(lib.spx_set_stream(self.h, C.c_void_p(s.cuda_stream)), self.h)

    def synchronize(self) -> None:
        self.bind_stream()
        check(lib.spx_synchronize(self.h), self.h)

    def check(self, status: int) -> None:
        check(status, self.h)


_contexts: dict[int, Context] = {}


def default_context(device: int | None = None) -> Context:
    torch = _torch()
    d = torch.cuda.current_device() if device is None else int(device)
    if d not in _contexts:
        _contexts[d] = Context(d)
    return _contexts[d]


def _ctx_for(t, ctx):
    ctx = ctx or default_context(t.device.index)
    ctx.bind_stream()
    return ctx


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _require_cuda(t, dtype, name):
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise ValueError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


def maxvalues_to_numpy(t) -> np.ndarray:
    """[..., 8] int32 words (device or host) -> numpy structured MaxValue array [...]."""
    a = t.detach().cpu().contiguous().numpy()
    return a.view(MAXVALUE_DTYPE)[..., 0]


def fft(x, nfft: int | None = None, window: int = WINDOW_NONE, out: str = "complex",
        scale: float = 1.0, ctx: Context | None = None):
    """Windowed, zero-padded batched FFT of x [beams, n_point] complex64."""
    torch = _torch()
    _require_cuda(x, torch.complex64, "x")
    x2 = x.reshape(-1, x.shape[-1])
    beams, n_point = x2.shape
    nfft = int(nfft or n_point)
    mode = _OUT_MODES[out]
    if not 0 < nfft <= 0xFFFFFFFF or not lib.spx_fft_size_supported(nfft):
        raise ValueError(f"spx_fft: nfft={nfft} is not a transform size of this build")
    shape = (beams, nfft)
    if mode == OUT_COMPLEX:
        o = torch.empty(shape, dtype=torch.complex64, device=x.device)
    elif mode == OUT_MAGPHASE:
        o = torch.empty(shape + (2,), dtype=torch.float32, device=x.device)
    else:
        o = torch.empty(shape, dtype=torch.float32, device=x.device)
    c = _ctx_for(x, ctx)
    c.check(lib.spx_fft(c.h, _ptr(x2), beams, n_point, nfft, window, mode, scale, _ptr(o)))
    return o


def ifft(spec, out=None, ctx: Context | None = None):
    """Inverse FFT with 1/nfft scaling of spec [beams, nfft] complex64 (CpuFFT::InverseC2C)."""
    torch = _torch()
    _require_cuda(spec, torch.complex64, "spec")
    s2 = spec.reshape(-1, spec.shape[-1])
    beams, nfft = s2.shape
    o = torch.empty_like(s2) if out is None else out
    c = _ctx_for(spec, ctx)
    c.check(lib.spx_ifft(c.h, _ptr(s2), beams, nfft, _ptr(o)))
    return o.reshape(spec.shape)


def fft_r2c(x, nfft: int | None = None, window: int = WINDOW_NONE, full: bool = False,
            ctx: Context | None = None):
    """FFT of real x [beams, n_point] float32 -> complex64 [beams, nfft/2 + 1]
    (CpuFFT::ForwardR2C) or [beams, nfft] with the conjugate mirror (full)."""
    torch = _torch()
    _require_cuda(x, torch.float32, "x")
    x2 = x.reshape(-1, x.shape[-1])
    beams, n_point = x2.shape
    nfft = int(nfft or n_point)
    o = torch.empty((beams, nfft if full else nfft // 2 + 1), dtype=torch.complex64, device=x.device)
    c = _ctx_for(x, ctx)
    c.check(lib.spx_fft_r2c(c.h, _ptr(x2), beams, n_point, nfft, window, 1 if full else 0, _ptr(o)))
    return o


def magnitude(z, inv_n: float = 1.0, squared: bool = False, ctx: Context | None = None):
    torch = _torch()
    _require_cuda(z, torch.complex64, "z")
    o = torch.empty(z.shape, dtype=torch.float32, device=z.device)
    c = _ctx_for(z, ctx)
    c.check(lib.spx_magnitude(c.h, _ptr(z), _ptr(o), z.numel(), inv_n, int(squared)))
    return o


def mag_phase(z, ctx: Context | None = None):
    torch = _torch()
    _require_cuda(z, torch.complex64, "z")
    o = torch.empty(z.shape + (2,), dtype=torch.float32, device=z.device)
    c = _ctx_for(z, ctx)
    c.check(lib.spx_mag_phase(c.h, _ptr(z), _ptr(o), z.numel()))
    return o


def peaks_one_two(spec, search_range: int = 0, sample_rate: float = 1000.0, two: bool = False,
                  ctx: Context | None = None):
    """ONE_PEAK / TWO_PEAKS on a complex spectrum [beams, nfft] -> int32 [beams, 4|8, 8]."""
    torch = _torch()
    _require_cuda(spec, torch.complex64, "spec")
    beams, nfft = spec.reshape(-1, spec.shape[-1]).shape
    o = torch.empty((beams, 8 if two else 4, 8), dtype=torch.int32, device=spec.device)
    c = _ctx_for(spec, ctx)
    c.check(lib.spx_peaks_one_two(c.h, _ptr(spec), beams, nfft, search_range, sample_rate,
                                  int(two), _ptr(o)))
    return o


def all_maxima(spec, mag=None, sample_rate: float = 1000.0, search_start: int = 0,
               search_end: int = 0, max_per_beam: int = 1000, refine: int = REFINE_NONE,
               thresh_sigma: float = 0.0, ctx: Context | None = None):
    """All strict local maxima -> (int32 [beams, cap, 8] MaxValue words, uint32-as-int32 counts [beams])."""
    torch = _torch()
    _require_cuda(spec, torch.complex64, "spec")
    beams, nfft = spec.reshape(-1, spec.shape[-1]).shape
    if mag is not None:
        _require_cuda(mag, torch.float32, "mag")
    _, _, cap = _capi.all_maxima_capacity(nfft, search_start, search_end, max_per_beam)
    o = torch.empty((beams, max(cap, 0), 8), dtype=torch.int32, device=spec.device)
    counts = torch.empty(beams, dtype=torch.int32, device=spec.device)
    p = peak_params(PEAK_ALL, search_start, search_end, 0, max_per_beam, refine, sample_rate,
                    thresh_sigma)
    c = _ctx_for(spec, ctx)
    c.check(lib.spx_all_maxima(c.h, _ptr(mag), _ptr(spec), beams, nfft, C.byref(p), _ptr(o),
                               _ptr(counts)))
    return o, counts


def topk(spec, k: int, mag=None, sample_rate: float = 1000.0, search_start: int = 0,
         search_end: int = 0, refine: int = REFINE_PARABOLIC, thresh_sigma: float = 0.0,
         ctx: Context | None = None):
    """Top-K strict local maxima -> (int32 [beams, K, 8], counts [beams])."""
    torch = _torch()
    _require_cuda(spec, torch.complex64, "spec")
    beams, nfft = spec.reshape(-1, spec.shape[-1]).shape
    if mag is not None:
        _require_cuda(mag, torch.float32, "mag")
    o = torch.zeros((beams, k, 8), dtype=torch.int32, device=spec.device)
    counts = torch.empty(beams, dtype=torch.int32, device=spec.device)
    p = peak_params(PEAK_TOPK, search_start, search_end, 0, k, refine, sample_rate, thresh_sigma)
    c = _ctx_for(spec, ctx)
    c.check(lib.spx_topk(c.h, _ptr(mag), _ptr(spec), beams, nfft, C.byref(p), _ptr(o), _ptr(counts)))
    return o, counts


def fft_peaks(x, nfft: int, window: int = WINDOW_NONE, mode: int = PEAK_ALL,
              sample_rate: float = 1000.0, search_start: int = 0, search_end: int = 0,
              search_range: int = 0, max_per_beam: int = 1000, refine: int = REFINE_NONE,
              thresh_sigma: float = 0.0, ctx: Context | None = None):
    """Raw samples [beams, n_point] -> peaks in one call (layouts as the peak functions)."""
    torch = _torch()
    _require_cuda(x, torch.complex64, "x")
    x2 = x.reshape(-1, x.shape[-1])
    beams, n_point = x2.shape
    if mode in (PEAK_ONE, PEAK_TWO):
        per = 4 if mode == PEAK_ONE else 8
    elif mode == PEAK_ALL:
        per = _capi.all_maxima_capacity(nfft, search_start, search_end, max_per_beam)[2]
    else:
        per = max_per_beam
    o = torch.zeros((beams, per, 8), dtype=torch.int32, device=x.device)
    counts = torch.zeros(beams, dtype=torch.int32, device=x.device)
    p = peak_params(mode, search_start, search_end, search_range, max_per_beam, refine,
                    sample_rate, thresh_sigma)
    c = _ctx_for(x, ctx)
    c.check(lib.spx_fft_peaks(c.h, _ptr(x2), beams, n_point, nfft, window, C.byref(p), _ptr(o),
                              _ptr(counts)))
    return o, counts


def fft_peaks_host(x, nfft: int, window: int = WINDOW_NONE, mode: int = PEAK_ALL,
                   sample_rate: float = 1000.0, search_start: int = 0, search_end: int = 0,
                   search_range: int = 0, max_per_beam: int = 1000, refine: int = REFINE_NONE,
                   thresh_sigma: float = 0.0, out=None, counts=None, ctx: Context | None = None):
    """Host samples [beams, n_point] complex64 (numpy array or CPU tensor;
    page-locked memory overlaps the copies) -> host peaks, via
    spx_fft_peaks_host.  Returns (int32 [beams, R, 8] MaxValue words, counts
    [beams]) as CPU tensors, written into out / counts when given."""
    torch = _torch()
    if isinstance(x, np.ndarray):
        x = torch.from_numpy(np.ascontiguousarray(x, dtype=np.complex64))
    if x.is_cuda or x.dtype != torch.complex64 or not x.is_contiguous():
        raise ValueError("x must be a contiguous host complex64 tensor or array")
    x2 = x.reshape(-1, x.shape[-1])
    beams, n_point = x2.shape
    if mode in (PEAK_ONE, PEAK_TWO):
        per = 4 if mode == PEAK_ONE else 8
    elif mode == PEAK_ALL:
        per = _capi.all_maxima_capacity(nfft, search_start, search_end, max_per_beam)[2]
    else:
        per = max_per_beam
    if out is None:
        out = torch.zeros((beams, per, 8), dtype=torch.int32)
    if counts is None:
        counts = torch.zeros(beams, dtype=torch.int32)
    if out.is_cuda or out.numel() < beams * per * 8 or counts.is_cuda or counts.numel() < beams:
        raise ValueError("out / counts must be host tensors of [beams, R, 8] / [beams]")
    p = peak_params(mode, search_start, search_end, search_range, max_per_beam, refine,
                    sample_rate, thresh_sigma)
    c = ctx or default_context()
    c.bind_stream()
    c.check(lib.spx_fft_peaks_host(c.h, _ptr(x2), beams, n_point, nfft, window, C.byref(p), _ptr(out),
                                   _ptr(counts)))
    return out, counts


def next_pow2(n: int) -> int:
    return int(lib.spx_next_pow2(n))


def next_smooth23(n: int) -> int:
    return int(lib.spx_next_smooth23(n))


def fft_size_supported(nfft: int) -> bool:
    return bool(lib.spx_fft_size_supported(nfft))
