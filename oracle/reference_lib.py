"""ctypes access to oracle/_ref (the reference's own CPU FFT and kernel text,
built by oracle/build_ref.py).  TEST INFRASTRUCTURE ONLY; available only
where the reference sources were present at build time."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .spectrum_oracle import MAXVALUE_DTYPE

REF_DIR = Path(__file__).resolve().parent / "_ref"


def available() -> bool:
    return (REF_DIR / "libref_cpufft.so").exists() and (REF_DIR / "libref_kernels.so").exists()


_libs: dict = {}


def _lib(name):
    if name not in _libs:
        lib = C.CDLL(str(REF_DIR / f"libref_{name}.so"))
        if name == "kernels":
            lib.ref_post_peaks.argtypes = [C.c_void_p, C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_float, C.c_int]
            lib.ref_compute_magnitudes.argtypes = [C.c_void_p, C.c_void_p, C.c_uint]
            lib.ref_all_maxima.argtypes = [C.c_void_p, C.c_void_p, C.c_uint, C.c_uint, C.c_float, C.c_uint,
                                           C.c_uint, C.c_uint, C.c_void_p, C.c_void_p]
            lib.ref_all_maxima.restype = C.c_uint
            lib.ref_complex_to_magnitude.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_uint, C.c_int]
            lib.ref_complex_to_mag_phase.argtypes = [C.c_void_p, C.c_void_p, C.c_uint]
            lib.ref_pad_windowed.argtypes = [C.c_void_p, C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_int]
        else:
            lib.ref_cpu_fft_c2c.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t]
            lib.ref_cpu_ifft_c2c.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t]
            lib.ref_cpu_fft_r2c.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_int]
            lib.ref_cpu_magnitude.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        _libs[name] = lib
    return _libs[name]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def cpu_fft_c2c(x: np.ndarray) -> np.ndarray:
    """CpuFFT::ForwardC2C row by row."""
    x = np.ascontiguousarray(np.atleast_2d(x), np.complex64)
    out = np.empty_like(x)
    _lib("cpufft").ref_cpu_fft_c2c(_p(x), _p(out), x.shape[0], x.shape[1])
    return out


def cpu_ifft_c2c(x: np.ndarray) -> np.ndarray:
    """CpuFFT::InverseC2C (1/N) row by row."""
    x = np.ascontiguousarray(np.atleast_2d(x), np.complex64)
    out = np.empty_like(x)
    _lib("cpufft").ref_cpu_ifft_c2c(_p(x), _p(out), x.shape[0], x.shape[1])
    return out


def cpu_fft_r2c(x: np.ndarray, full: bool = False) -> np.ndarray:
    """CpuFFT::ForwardR2C (n/2 + 1 bins) or ForwardR2C_Full (n bins) row by row."""
    x = np.ascontiguousarray(np.atleast_2d(x), np.float32)
    n = x.shape[1]
    out = np.empty((x.shape[0], n if full else n // 2 + 1), np.complex64)
    _lib("cpufft").ref_cpu_fft_r2c(_p(x), _p(out), x.shape[0], n, 1 if full else 0)
    return out


def post_peaks(fft: np.ndarray, nfft: int, search_range: int, fs: float, two: bool) -> np.ndarray:
    fft = np.ascontiguousarray(fft, np.complex64).reshape(-1, nfft)
    if search_range == 0:
        search_range = nfft // 4  # CalculateFFTSize default (spectrum_processor_rocm.cpp:1137-1143)
    out = np.zeros((fft.shape[0], 8 if two else 4), MAXVALUE_DTYPE)
    _lib("kernels").ref_post_peaks(_p(fft), _p(out), fft.shape[0], nfft, search_range, fs, int(two))
    return out


def compute_magnitudes(fft: np.ndarray) -> np.ndarray:
    fft = np.ascontiguousarray(fft, np.complex64)
    out = np.empty(fft.shape, np.float32)
    _lib("kernels").ref_compute_magnitudes(_p(fft), _p(out), fft.size)
    return out


def all_maxima(mag: np.ndarray, fft: np.ndarray, nfft: int, fs: float, start=0, end=0, max_per_beam=1000):
    fft = np.ascontiguousarray(fft, np.complex64).reshape(-1, nfft)
    mag = np.ascontiguousarray(mag, np.float32).reshape(-1, nfft)
    beams = fft.shape[0]
    # capacity is computed inside; allocate the largest it can be
    out = np.zeros((beams, max(max_per_beam, 1)), MAXVALUE_DTYPE)
    counts = np.zeros(beams, np.uint32)
    tmp = np.zeros(beams * max(max_per_beam, 1), MAXVALUE_DTYPE)
    cap = _lib("kernels").ref_all_maxima(_p(mag), _p(fft), beams, nfft, fs, start, end, max_per_beam,
                                          _p(tmp), _p(counts))
    out = tmp[: beams * cap].reshape(beams, cap) if cap else np.zeros((beams, 0), MAXVALUE_DTYPE)
    return out, counts


def complex_to_magnitude(z: np.ndarray, inv_n=1.0, squared=False) -> np.ndarray:
    z = np.ascontiguousarray(z, np.complex64)
    out = np.empty(z.shape, np.float32)
    _lib("kernels").ref_complex_to_magnitude(_p(z), _p(out), inv_n, z.size, int(squared))
    return out


def complex_to_mag_phase(z: np.ndarray) -> np.ndarray:
    z = np.ascontiguousarray(z, np.complex64)
    out = np.empty(z.shape + (2,), np.float32)
    _lib("kernels").ref_complex_to_mag_phase(_p(z), _p(out), z.size)
    return out


def pad_windowed(x: np.ndarray, nfft: int, window: int) -> np.ndarray:
    x = np.ascontiguousarray(np.atleast_2d(x), np.complex64)
    out = np.empty((x.shape[0], nfft), np.complex64)
    _lib("kernels").ref_pad_windowed(_p(x), _p(out), x.shape[0], x.shape[1], nfft, window)
    return out
