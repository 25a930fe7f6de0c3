"""Python mirror of the reference's ``dsp_spectrum`` module for the FFT -> peaks
path: the same class names, method names, keyword arguments, defaults and
return shapes as its pybind11 classes, running on the C ABI of this library.

    import spectrum_gb300.dsp_spectrum as dsp_spectrum
    ctx = dsp_spectrum.ROCmGPUContext(device_index=0)
    fft = dsp_spectrum.FFTProcessorROCm(ctx)
    spec = fft.process_complex(data, sample_rate=1e6)
    finder = dsp_spectrum.SpectrumMaximaFinderROCm(ctx)
    peaks = finder.process(signal, n_point=1000, sample_rate=10e3)

Mirrored (python/dsp_spectrum_module.cpp:35-68):
  ROCmGPUContext            (device_index, device_name)
  FFTProcessorROCm          python/py_fft_processor_rocm.hpp:30-225
  SpectrumMaximaFinderROCm  python/py_spectrum_maxima_finder_rocm.hpp:39-336
  ComplexToMagROCm          python/py_complex_to_mag_rocm.hpp:42-147
Inputs are numpy arrays (cast to complex64, C order) like the pybind11
``forcecast`` arrays; outputs are numpy arrays / dicts as there.  Invalid
arguments raise ValueError (std::invalid_argument); device failures
RuntimeError.  There is no CPU path: without the native library or a GPU the
constructors raise.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import MAXVALUE_DTYPE, Context
from ._capi import (OUT_COMPLEX, OUT_MAGPHASE, PEAK_ALL, PEAK_ONE, REFINE_NONE, REFINE_PARABOLIC,
                    WINDOW_NONE, lib, peak_params)


def _c64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex64)


def _shape(buf: np.ndarray, beams: int, n_point: int = 0):
    total = buf.size
    if buf.ndim == 2:
        beams = beams or buf.shape[0]
        n_point = n_point or buf.shape[1]
    else:
        beams = beams or 1
        n_point = n_point or (total // beams)
    if beams == 0 or n_point == 0 or total != beams * n_point:
        raise ValueError(f"data of {total} samples is not beam_count={beams} x n_point={n_point}")
    return beams, n_point


def _nfft(n_point: int, repeat_count: int) -> int:
    if n_point == 0 or repeat_count == 0:
        raise ValueError("n_point and repeat_count must be > 0")
    n = int(lib.spx_next_pow2(n_point)) * int(repeat_count)
    if n > 0xFFFFFFFF or not lib.spx_fft_size_supported(n):
        raise ValueError(f"nFFT {n} is not a transform size of this build")
    return n


class ROCmGPUContext:
    """Device context handed to the processors (the reference's ROCmGPUContext)."""

    def __init__(self, device_index: int = 0):
        import torch
        self._ctx = Context(device_index)
        self._device = torch.device("cuda", int(device_index))

    @property
    def device_index(self) -> int:
        return self._ctx.device

    @property
    def device_name(self) -> str:
        import torch
        return torch.cuda.get_device_name(self._ctx.device)

    def _bind(self):
        self._ctx.bind_stream()
        return self._ctx

    def __repr__(self) -> str:
        return f"<ROCmGPUContext device_index={self.device_index}>"


GPUContext = ROCmGPUContext


class FFTProcessorROCm:
    def __init__(self, ctx: ROCmGPUContext):
        self._c = ctx
        self._nfft = 0
        self._prof = {"upload_ms": 0.0, "fft_ms": 0.0, "post_processing_ms": 0.0, "download_ms": 0.0,
                      "total_ms": 0.0}

    @property
    def nfft(self) -> int:
        return self._nfft

    def _run(self, data, beam_count, n_point, out_mode):
        import torch
        x = _c64(data)
        beams, n_point = _shape(x, beam_count, n_point)
        nfft = _nfft(n_point, 1)
        self._nfft = nfft
        ctx = self._c._bind()
        stream = torch.cuda.current_stream(self._c._device)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ev[0].record(stream)
        xd = torch.from_numpy(x.reshape(beams, n_point)).to(self._c._device, non_blocking=False)
        ev[1].record(stream)
        out = torch.empty((beams, nfft), dtype=torch.complex64, device=self._c._device)
        ctx.check(lib.spx_fft(ctx.h, C.c_void_p(xd.data_ptr()), beams, n_point, nfft, WINDOW_NONE, out_mode,
                              1.0, C.c_void_p(out.data_ptr())))
        ev[2].record(stream)
        host = out.cpu()
        ev[3].record(stream)
        torch.cuda.synchronize(self._c._device)
        self._prof = {"upload_ms": ev[0].elapsed_time(ev[1]), "fft_ms": ev[1].elapsed_time(ev[2]),
                      "post_processing_ms": 0.0, "download_ms": ev[2].elapsed_time(ev[3]),
                      "total_ms": ev[0].elapsed_time(ev[3])}
        return host.numpy(), beams, nfft

    def process_complex(self, data, sample_rate: float, beam_count: int = 0, n_point: int = 0) -> np.ndarray:
        """-> complex64 (nFFT,) for one beam, (beam_count, nFFT) otherwise."""
        spec, beams, _ = self._run(data, beam_count, n_point, OUT_COMPLEX)
        return spec[0].copy() if beams == 1 else spec

    def process_mag_phase(self, data, sample_rate: float, beam_count: int = 0, n_point: int = 0,
                          include_freq: bool = True) -> dict:
        """-> dict(magnitude, phase[, frequency], nFFT, sample_rate)."""
        raw, beams, nfft = self._run(data, beam_count, n_point, OUT_MAGPHASE)
        mp = raw.view(np.float32).reshape(beams, nfft, 2)
        out = {"nFFT": nfft, "sample_rate": float(np.float32(sample_rate))}
        mag, ph = np.ascontiguousarray(mp[..., 0]), np.ascontiguousarray(mp[..., 1])
        freq = None
        if include_freq:  # fft_processor_rocm.cpp:289-295
            step = np.float32(sample_rate) / np.float32(nfft)
            freq = np.broadcast_to(np.arange(nfft, dtype=np.float32) * step, (beams, nfft)).copy()
        if beams == 1:
            out["magnitude"], out["phase"] = mag[0], ph[0]
            if freq is not None:
                out["frequency"] = freq[0]
        else:
            out["magnitude"], out["phase"] = mag, ph
            if freq is not None:
                out["frequency"] = freq
        return out

    def get_profiling(self) -> dict:
        return dict(self._prof)

    def __repr__(self) -> str:
        return f"<FFTProcessorROCm nfft={self._nfft}>"


class ComplexToMagROCm:
    def __init__(self, ctx: ROCmGPUContext):
        self._c = ctx

    def process_magnitude(self, data, beam_count: int = 0, norm_coeff: float = 1.0) -> np.ndarray:
        """|z| x inv_n (norm_coeff 0: x1, -1: /n_point, > 0: x norm_coeff)."""
        import torch
        x = _c64(data)
        if x.ndim == 2 and beam_count == 0:
            beam_count = x.shape[0]
        beam_count = beam_count or 1
        total = x.size
        if total % beam_count:
            raise ValueError(f"process_magnitude: total={total} not divisible by beam_count={beam_count}")
        n_point = total // beam_count
        if norm_coeff < 0:
            inv_n = 1.0 / n_point if n_point > 0 else 1.0
        elif norm_coeff > 0:
            inv_n = norm_coeff
        else:
            inv_n = 1.0
        ctx = self._c._bind()
        xd = torch.from_numpy(x.reshape(-1)).to(self._c._device)
        out = torch.empty(total, dtype=torch.float32, device=self._c._device)
        ctx.check(lib.spx_magnitude(ctx.h, C.c_void_p(xd.data_ptr()), C.c_void_p(out.data_ptr()), total,
                                    float(np.float32(inv_n)), 0))
        m = out.cpu().numpy()
        return m if beam_count == 1 else m.reshape(beam_count, n_point)

    def __repr__(self) -> str:
        return "<ComplexToMagROCm>"


class SpectrumMaximaFinderROCm:
    def __init__(self, ctx: ROCmGPUContext):
        self._c = ctx
        self._params = None

    def _init(self, antenna_count, n_point, sample_rate, repeat_count, mode):
        nfft = _nfft(n_point, repeat_count)
        self._params = {"antenna_count": antenna_count, "n_point": n_point, "repeat_count": repeat_count,
                        "sample_rate": float(np.float32(sample_rate)), "nFFT": nfft, "peak_mode": mode}
        return nfft

    def is_initialized(self) -> bool:
        return self._params is not None

    def get_params(self) -> dict:
        if self._params is None:
            return {"antenna_count": 0, "n_point": 0, "repeat_count": 0, "sample_rate": 0.0, "nFFT": 0}
        return {k: v for k, v in self._params.items() if k != "peak_mode"}

    def _host_call(self, x, beams, n_point, nfft, p, per):
        out = np.zeros((beams, per), dtype=MAXVALUE_DTYPE)
        counts = np.zeros(beams, dtype=np.uint32)
        ctx = self._c._bind()
        ctx.check(lib.spx_fft_peaks_host(ctx.h, x.ctypes.data_as(C.c_void_p), beams, n_point, nfft, WINDOW_NONE,
                                         C.byref(p), out.ctypes.data_as(C.c_void_p),
                                         counts.ctypes.data_as(C.c_void_p)))
        return out, counts

    def process(self, signal, n_point: int, sample_rate: float, antenna_count: int = 0, repeat_count: int = 1):
        """ONE_PEAK per antenna -> dict (one antenna) or list of dicts with
        antenna_id, freq_hz, magnitude, phase (degrees), index, freq_offset."""
        x = _c64(signal)
        if antenna_count == 0:
            antenna_count = x.shape[0] if x.ndim == 2 else 1
        if x.size != antenna_count * n_point:
            raise ValueError(f"input size mismatch. Expected {antenna_count * n_point}, got {x.size}")
        nfft = self._init(antenna_count, n_point, sample_rate, repeat_count, "ONE_PEAK")
        p = peak_params(PEAK_ONE, 0, 0, nfft // 4, 0, REFINE_PARABOLIC, sample_rate, 0.0)
        out, _ = self._host_call(x, antenna_count, n_point, nfft, p, 4)
        res = [{"antenna_id": b, "freq_hz": float(out[b, 0]["refined_frequency"]),
                "magnitude": float(out[b, 0]["magnitude"]), "phase": float(out[b, 0]["phase"]),
                "index": int(out[b, 0]["index"]), "freq_offset": float(out[b, 0]["freq_offset"])}
               for b in range(antenna_count)]
        return res[0] if len(res) == 1 else res

    @staticmethod
    def _all_result(out, counts, cap, beams):
        res = []
        for b in range(beams):
            n = int(min(counts[b], cap))
            m = out[b, :n]
            res.append({"antenna_id": b, "positions": m["index"].astype(np.uint32).copy(),
                        "magnitudes": m["magnitude"].copy(), "frequencies": m["refined_frequency"].copy(),
                        "num_maxima": n})
        return res[0] if beams == 1 and len(res) == 1 else res

    def find_all_maxima(self, fft_data, nFFT: int, sample_rate: float, beam_count: int = 0,  # noqa: N803
                        search_start: int = 0, search_end: int = 0):
        """All strict local maxima of |X| on spectra already computed."""
        import torch
        x = _c64(fft_data)
        if beam_count == 0:
            beam_count = x.shape[0] if x.ndim == 2 else 1
        if x.size != beam_count * nFFT:
            raise ValueError(f"fft_data size {x.size} != beam_count * nFFT {beam_count * nFFT}")
        self._init(beam_count, nFFT, sample_rate, 1, "ALL_MAXIMA")
        s, e, cap = C.c_uint32(), C.c_uint32(), C.c_uint32()
        lib.spx_all_maxima_capacity(nFFT, search_start, search_end, 1000, C.byref(s), C.byref(e), C.byref(cap))
        cap = cap.value
        ctx = self._c._bind()
        xd = torch.from_numpy(x.reshape(beam_count, nFFT)).to(self._c._device)
        od = torch.empty((beam_count, max(cap, 1), 8), dtype=torch.int32, device=self._c._device)
        cd = torch.empty(beam_count, dtype=torch.int32, device=self._c._device)
        p = peak_params(PEAK_ALL, search_start, search_end, 0, 1000, REFINE_NONE, sample_rate, 0.0)
        ctx.check(lib.spx_all_maxima(ctx.h, None, C.c_void_p(xd.data_ptr()), beam_count, nFFT, C.byref(p),
                                     C.c_void_p(od.data_ptr()), C.c_void_p(cd.data_ptr())))
        ctx.synchronize()
        out = od.cpu().numpy().view(MAXVALUE_DTYPE)[..., 0]
        return self._all_result(out, cd.cpu().numpy().astype(np.uint32), cap, beam_count)

    def find_all_maxima_from_signal(self, signal, n_point: int, sample_rate: float, antenna_count: int = 0,
                                    repeat_count: int = 1, search_start: int = 0, search_end: int = 0):
        """Signal -> pad + FFT + all strict local maxima (no window, no refinement)."""
        x = _c64(signal)
        if antenna_count == 0:
            antenna_count = x.shape[0] if x.ndim == 2 else 1
        if x.size != antenna_count * n_point:
            raise ValueError(f"input size mismatch. Expected {antenna_count * n_point}, got {x.size}")
        nfft = self._init(antenna_count, n_point, sample_rate, repeat_count, "ALL_MAXIMA")
        s, e, cap = C.c_uint32(), C.c_uint32(), C.c_uint32()
        lib.spx_all_maxima_capacity(nfft, search_start, search_end, 1000, C.byref(s), C.byref(e), C.byref(cap))
        p = peak_params(PEAK_ALL, search_start, search_end, 0, 1000, REFINE_NONE, sample_rate, 0.0)
        out, counts = self._host_call(x, antenna_count, n_point, nfft, p, max(cap.value, 1))
        return self._all_result(out, counts, cap.value, antenna_count)

    def __repr__(self) -> str:
        p = self._params or {}
        return f"<SpectrumMaximaFinderROCm nFFT={p.get('nFFT', 0)}>"
