"""Batches of beams with uneven lengths and FFT sizes (spx_batch_* of include/spx.h).

    b = Batch(n_points, window=WINDOW_HANN, k=8, sample_rate=fs)
    out, counts = b.run(x_packed)            # one FFT launch + one top-K launch
    out, counts = b.run_per_size(x_packed)   # the same kernel once per distinct nfft
    b.capture(x_packed); b.replay()          # CUDA graph of run() for fixed buffers
    b.autotune(x_packed)                     # per-size local FFT sizes, timed
    b.save_plans(path); b.load_plans(path)   # the plans as a JSON cache

x_packed holds the beams back to back (complex64, sum(n_points) samples).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import PEAK_TOPK, REFINE_PARABOLIC, WINDOW_NONE, lib


class Batch:
    def __init__(self, n_points, nffts=None, window: int = WINDOW_NONE, k: int = 8,
                 sample_rate: float = 1.0, refine: int = REFINE_PARABOLIC, search_start: int = 0,
                 search_end: int = 0, ctx=None):
        import torch

        from . import default_context
        self.ctx = ctx or default_context()
        self.n_points = np.ascontiguousarray(n_points, dtype=np.uint32)
        self.beams = len(self.n_points)
        self.k = int(k)
        nf = None if nffts is None else np.ascontiguousarray(nffts, dtype=np.uint32)
        p = _capi.peak_params(PEAK_TOPK, search_start, search_end, 0, k, refine, sample_rate, 0.0)
        h = C.c_void_p()
        self.ctx.bind_stream()
        self.ctx.check(lib.spx_batch_create(self.ctx.h, self.beams,
                                            self.n_points.ctypes.data_as(C.c_void_p),
                                            nf.ctypes.data_as(C.c_void_p) if nf is not None else None,
                                            window, C.byref(p), C.byref(h)))
        self.h = h
        self.nffts = [int(nf[i]) if nf is not None and nf[i] else int(_capi.lib.spx_next_smooth23(int(v)))
                      for i, v in enumerate(self.n_points)]
        dev = torch.device("cuda", self.ctx.device)
        self.out = torch.zeros((self.beams, self.k, 8), dtype=torch.int32, device=dev)
        self.counts = torch.zeros(self.beams, dtype=torch.int32, device=dev)

    @property
    def input_samples(self) -> int:
        return int(lib.spx_batch_input_samples(self.h))

    def _args(self, x):
        import torch
        if not (isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == torch.complex64 and x.is_contiguous()):
            raise ValueError("x must be a contiguous CUDA complex64 tensor")
        if x.numel() != self.input_samples:
            raise ValueError(f"x holds {x.numel()} samples, the batch needs {self.input_samples}")
        return (C.c_void_p(x.data_ptr()), C.c_void_p(self.out.data_ptr()), C.c_void_p(self.counts.data_ptr()))

    def run(self, x):
        self.ctx.bind_stream()
        self.ctx.check(lib.spx_batch_run(self.ctx.h, self.h, *self._args(x)))
        return self.out, self.counts

    def run_per_size(self, x):
        self.ctx.bind_stream()
        self.ctx.check(lib.spx_batch_run_per_size(self.ctx.h, self.h, *self._args(x)))
        return self.out, self.counts

    def capture(self, x, stream=None):
        self.ctx.bind_stream(stream)
        self.ctx.check(lib.spx_batch_capture(self.ctx.h, self.h, *self._args(x)))

    def replay(self, stream=None):
        self.ctx.bind_stream(stream)
        self.ctx.check(lib.spx_batch_replay(self.ctx.h, self.h))
        return self.out, self.counts

    def tune(self, points_per_thread: int, points_per_cta: int = 0):
        self.ctx.check(lib.spx_batch_tune(self.ctx.h, self.h, points_per_thread, points_per_cta))

    def autotune(self, x):
        """For every distinct nfft, times the whole batch with each candidate
        local FFT size of that nfft and keeps the fastest; returns (sizes
        tuned, plans changed)."""
        t, c = C.c_uint32(), C.c_uint32()
        self.ctx.bind_stream()
        self.ctx.check(lib.spx_batch_autotune(self.ctx.h, self.h, *self._args(x), C.byref(t), C.byref(c)))
        return t.value, c.value

    def local_size(self, nfft: int) -> int:
        """The local FFT size M of nfft's plan (C = nfft / M CTAs per beam)."""
        return int(lib.spx_batch_local_size(self.h, int(nfft)))

    def set_local_size(self, nfft: int, local_size: int):
        self.ctx.check(lib.spx_batch_set_local_size(self.ctx.h, self.h, int(nfft), int(local_size)))

    @property
    def cluster(self) -> int:
        """CTAs per cluster of the single FFT launch."""
        return int(lib.spx_batch_cluster(self.h))

    def set_cluster(self, cluster: int):
        """CTAs per cluster of the single FFT launch (0: the largest C the
        beams need; else that or more, up to 16)."""
        self.ctx.check(lib.spx_batch_set_cluster(self.ctx.h, self.h, int(cluster)))

    @property
    def plans(self) -> dict:
        """{nfft: local size} of the batch's distinct sizes."""
        return {int(n): self.local_size(int(n)) for n in sorted(set(self.nffts))}

    def save_plans(self, path):
        self.ctx.check(lib.spx_batch_save_plans(self.ctx.h, self.h, str(path).encode()))

    def load_plans(self, path) -> int:
        """Applies a saved plan file; returns the number of entries applied."""
        n = C.c_uint32()
        self.ctx.check(lib.spx_batch_load_plans(self.ctx.h, self.h, str(path).encode(), C.byref(n)))
        return n.value

    def close(self):
        if getattr(self, "h", None):
            lib.spx_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
