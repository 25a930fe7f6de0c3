"""ctypes binding of the C ABI declared in include/spx.h.

This is the same binding a ctypes user of the reference would add; every
entry point returns an ``spx_status`` that is turned into the exception type
the reference throws: ``ValueError`` (std::invalid_argument) for
SPX_ERR_INVALID_ARG, ``RuntimeError`` (std::runtime_error) otherwise.
There is no CPU fallback: importing this module without the built library
raises immediately.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "lib" / "libspectrum_gb300.so"

SPX_OK = 0
SPX_ERR_INVALID_ARG = 1
SPX_ERR_CUDA = 2
SPX_ERR_OUT_OF_MEMORY = 3
SPX_ERR_UNSUPPORTED = 4
SPX_ERR_TIMEOUT = 5
SPX_ERR_NO_DEVICE = 6

OUT_COMPLEX, OUT_MAG, OUT_MAG2, OUT_MAGPHASE = range(4)
WINDOW_NONE, WINDOW_HANN, WINDOW_HAMMING, WINDOW_BLACKMAN, WINDOW_BLACKMAN_HARRIS = range(5)
REFINE_NONE, REFINE_PARABOLIC = range(2)
PEAK_ONE, PEAK_TWO, PEAK_ALL, PEAK_TOPK = range(4)


class SpxMaxValue(C.Structure):
    _fields_ = [
        ("index", C.c_uint32),
        ("real", C.c_float),
        ("imag", C.c_float),
        ("magnitude", C.c_float),
        ("phase", C.c_float),
        ("freq_offset", C.c_float),
        ("refined_frequency", C.c_float),
        ("pad", C.c_uint32),
    ]


class SpxPeakParams(C.Structure):
    _fields_ = [
        ("mode", C.c_uint32),
        ("search_start", C.c_uint32),
        ("search_end", C.c_uint32),
        ("search_range", C.c_uint32),
        ("max_per_beam", C.c_uint32),
        ("refine", C.c_uint32),
        ("sample_rate", C.c_float),
        ("thresh_sigma", C.c_float),
    ]


assert C.sizeof(SpxMaxValue) == 32

_vp = C.c_void_p
_u32 = C.c_uint32
_u64 = C.c_uint64
_f = C.c_float
_i = C.c_int

# name -> (restype, argtypes); every symbol declared in include/spx.h.
PROTOTYPES: dict[str, tuple] = {
    "spx_create": (_i, [_i, C.POINTER(_vp)]),
    "spx_destroy": (_i, [_vp]),
    "spx_set_stream": (_i, [_vp, _vp]),
    "spx_get_stream": (_vp, [_vp]),
    "spx_synchronize": (_i, [_vp]),
    "spx_last_error": (C.c_char_p, [_vp]),
    "spx_status_string": (C.c_char_p, [_i]),
    "spx_abi_version": (_i, []),
    "spx_scratch_bytes": (_u64, [_vp]),
    "spx_selftest_wait_timeout": (_i, [_vp]),
    "spx_selftest_group_wait_timeout": (_i, [_vp]),
    "spx_next_pow2": (_u32, [_u32]),
    "spx_next_smooth23": (_u32, [_u32]),
    "spx_fft_size_supported": (_i, [_u32]),
    "spx_set_fft_tuning": (_i, [_vp, _u32, _u32, _u32]),
    "spx_all_maxima_capacity": (_i, [_u32, _u32, _u32, _u32, C.POINTER(_u32), C.POINTER(_u32), C.POINTER(_u32)]),
    "spx_noise_threshold_factor": (_f, [_f]),
    "spx_fft": (_i, [_vp, _vp, _u32, _u32, _u32, _u32, _u32, _f, _vp]),
    "spx_ifft": (_i, [_vp, _vp, _u32, _u32, _vp]),
    "spx_fft_r2c": (_i, [_vp, _vp, _u32, _u32, _u32, _u32, _i, _vp]),
    "spx_magnitude": (_i, [_vp, _vp, _vp, _u64, _f, _i]),
    "spx_mag_phase": (_i, [_vp, _vp, _vp, _u64]),
    "spx_peaks_one_two": (_i, [_vp, _vp, _u32, _u32, _u32, _f, _i, _vp]),
    "spx_all_maxima": (_i, [_vp, _vp, _vp, _u32, _u32, C.POINTER(SpxPeakParams), _vp, _vp]),
    "spx_topk": (_i, [_vp, _vp, _vp, _u32, _u32, C.POINTER(SpxPeakParams), _vp, _vp]),
    "spx_fft_peaks": (_i, [_vp, _vp, _u32, _u32, _u32, _u32, C.POINTER(SpxPeakParams), _vp, _vp]),
    "spx_all_maxima_noalloc": (_i, [_vp, _vp, _vp, _u32, _u32, C.POINTER(SpxPeakParams), _vp, _vp]),
    "spx_fft_peaks_host": (_i, [_vp, _vp, _u32, _u32, _u32, _u32, C.POINTER(SpxPeakParams), _vp, _vp]),
    "spx_batch_create": (_i, [_vp, _u32, _vp, _vp, _u32, C.POINTER(SpxPeakParams), C.POINTER(_vp)]),
    "spx_batch_destroy": (_i, [_vp]),
    "spx_batch_input_samples": (_u64, [_vp]),
    "spx_batch_run": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "spx_batch_run_per_size": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "spx_batch_capture": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "spx_batch_replay": (_i, [_vp, _vp]),
    "spx_batch_tune": (_i, [_vp, _vp, _u32, _u32]),
    "spx_batch_local_size": (_u32, [_vp, _u32]),
    "spx_batch_set_local_size": (_i, [_vp, _vp, _u32, _u32]),
    "spx_batch_cluster": (_u32, [_vp]),
    "spx_batch_set_cluster": (_i, [_vp, _vp, _u32]),
    "spx_batch_autotune": (_i, [_vp, _vp, _vp, _vp, _vp, C.POINTER(_u32), C.POINTER(_u32)]),
    "spx_batch_save_plans": (_i, [_vp, _vp, C.c_char_p]),
    "spx_batch_load_plans": (_i, [_vp, _vp, C.c_char_p, C.POINTER(_u32)]),
    "spx_mlp_param_count": (_u32, []),
    "spx_mlp_create": (_i, [_vp, _u64, C.POINTER(_vp)]),
    "spx_mlp_destroy": (_i, [_vp]),
    "spx_mlp_set_params": (_i, [_vp, _vp, _vp]),
    "spx_mlp_get_params": (_i, [_vp, _vp, _vp]),
    "spx_mlp_make_frames": (_i, [_vp, _u64, _u32, _u32, _u32, _f, _f, _vp, _vp, _vp, _vp, _vp]),
    "spx_mlp_forward": (_i, [_vp, _vp, _vp, _u32, _vp]),
    "spx_mlp_gradients": (_i, [_vp, _vp, _vp, _vp, _vp, _u32, _vp, _vp]),
    "spx_mlp_train_step": (_i, [_vp, _vp, _vp, _vp, _vp, _u32, _f, _vp]),
    "spx_mlp_train": (_i, [_vp, _vp, _vp, _vp, _vp, _u32, _u32, _u32, _f, _f, _u64, _vp]),
    "spx_mlp_refine": (_i, [_vp, _vp, _vp, _u32, _u32, _u32, _f, _u32, _vp, _vp, _vp, _vp]),
    "spx_fft_peaks_mlp": (_i, [_vp, _vp, _vp, _u32, _u32, _u32, _u32, _vp, _vp, _vp, _vp, _vp]),
}


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    p = Path(path) if path else _LIB_PATH
    if not p.exists():
        raise ImportError(
            f"spectrum_gb300 native library not found at {p}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = load_library()


class SpxError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{lib.spx_status_string(status).decode()}: {msg}")
        self.status = status


class SpxInvalidArgument(SpxError, ValueError):
    pass


def check(status: int, ctx=None) -> None:
    if status == SPX_OK:
        return
    msg = lib.spx_last_error(ctx).decode() if ctx else ""
    if status == SPX_ERR_INVALID_ARG:
        raise SpxInvalidArgument(status, msg)
    raise SpxError(status, msg)


def peak_params(mode=PEAK_ALL, search_start=0, search_end=0, search_range=0, max_per_beam=1000,
                refine=REFINE_NONE, sample_rate=1000.0, thresh_sigma=0.0) -> SpxPeakParams:
    return SpxPeakParams(mode, search_start, search_end, search_range, max_per_beam, refine,
                         sample_rate, thresh_sigma)


def all_maxima_capacity(nfft: int, start: int = 0, end: int = 0, max_per_beam: int = 1000):
    s, e, c = _u32(), _u32(), _u32()
    st = lib.spx_all_maxima_capacity(nfft, start, end, max_per_beam, C.byref(s), C.byref(e), C.byref(c))
    check(st)
    return s.value, e.value, c.value
