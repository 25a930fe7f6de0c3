"""Learned sub-bin refinement (spx_mlp_* of include/spx.h).

A 10 -> 64 -> 64 -> 2 GELU network (BF16 weights, FP32 accumulation) that
maps the 5 bins around a spectral peak to the tone's offset from the bin and
its amplitude correction.  Everything runs on the GPU through the native
library: training frames are made by the library's own FFT, the labels come
from a 16x zero-padded FFT of the same frames, and forward, backward and Adam
are hand-written kernels.

    r = MLPRefiner(seed=1)
    data = r.make_frames(1 << 20, nfft=1024, snr_db=(0, 40), seed=7)
    losses = r.train(data, epochs=20, batch=4096)
    out, counts = spectrum_gb300.topk(spec, 1, sample_rate=fs)   # parabolic
    amp, used = r.refine(spec, out, counts, n_point, fs)           # learned
    r.save("refiner.spxmlp"); r2 = MLPRefiner.load("refiner.spxmlp")

File format (``save``/``load``): 8-byte magic ``b"SPXMLP1\\n"``, uint32
little-endian header length, a JSON header naming the layers and tensor
layout, then the tensors back to back: weights as BF16, biases as FP32 (the
exact values inference uses).
"""
from __future__ import annotations

import ctypes as C
import json
import struct

import numpy as np

from . import _capi
from ._capi import lib

N_IN, N_HIDDEN, N_OUT = 10, 64, 2
N_PARAMS = int(lib.spx_mlp_param_count())
# (name, shape, file dtype) in parameter order
LAYOUT = [("W1", (N_HIDDEN, N_IN), "bf16"), ("b1", (N_HIDDEN,), "f32"),
          ("W2", (N_HIDDEN, N_HIDDEN), "bf16"), ("b2", (N_HIDDEN,), "f32"),
          ("W3", (N_OUT, N_HIDDEN), "bf16"), ("b3", (N_OUT,), "f32")]
assert sum(int(np.prod(s)) for _, s, _ in LAYOUT) == N_PARAMS
MAGIC = b"SPXMLP1\n"


def bf16_round(x: np.ndarray) -> np.ndarray:
    """FP32 -> nearest BF16 (ties to even), returned as FP32 values."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class MLPRefiner:
    def __init__(self, seed: int = 0, ctx=None):
        from . import default_context
        self.ctx = ctx or default_context()
        h = C.c_void_p()
        self.ctx.bind_stream()
        self.ctx.check(lib.spx_mlp_create(self.ctx.h, int(seed), C.byref(h)))
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            lib.spx_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- parameters --------------------------------------------------------
    @property
    def params(self) -> np.ndarray:
        p = np.empty(N_PARAMS, np.float32)
        self.ctx.bind_stream()
        self.ctx.check(lib.spx_mlp_get_params(self.ctx.h, self.h, p.ctypes.data_as(C.c_void_p)))
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.shape != (N_PARAMS,):
            raise ValueError(f"expected {N_PARAMS} parameters, got shape {p.shape}")
        self.ctx.bind_stream()
        self.ctx.check(lib.spx_mlp_set_params(self.ctx.h, self.h, p.ctypes.data_as(C.c_void_p)))

    def save(self, path) -> None:
        p = self.params
        header = {"format": "spx-mlp", "version": 1, "layers": [N_IN, N_HIDDEN, N_HIDDEN, N_OUT],
                  "activation": "gelu-erf",
                  "tensors": [{"name": n, "shape": list(s), "dtype": d} for n, s, d in LAYOUT]}
        hb = json.dumps(header).encode()
        chunks, off = [], 0
        for _, shape, dt in LAYOUT:
            n = int(np.prod(shape))
            v = p[off:off + n]
            off += n
            if dt == "bf16":
                chunks.append((bf16_round(v).view(np.uint32) >> 16).astype("<u2").tobytes())
            else:
                chunks.append(v.astype("<f4").tobytes())
        with open(path, "wb") as f:
            f.write(MAGIC + struct.pack("<I", len(hb)) + hb + b"".join(chunks))

    @classmethod
    def load(cls, path, ctx=None) -> "MLPRefiner":
        with open(path, "rb") as f:
            blob = f.read()
        if blob[:8] != MAGIC:
            raise ValueError(f"{path}: not an spx-mlp file")
        (hl,) = struct.unpack("<I", blob[8:12])
        header = json.loads(blob[12:12 + hl])
        if header.get("layers") != [N_IN, N_HIDDEN, N_HIDDEN, N_OUT]:
            raise ValueError(f"{path}: layer sizes {header.get('layers')} are not 10-64-64-2")
        pos, parts = 12 + hl, []
        for t, (name, shape, dt) in zip(header["tensors"], LAYOUT):
            if t["name"] != name or tuple(t["shape"]) != shape or t["dtype"] != dt:
                raise ValueError(f"{path}: unexpected tensor entry {t}")
            n = int(np.prod(shape))
            if dt == "bf16":
                raw = np.frombuffer(blob, "<u2", n, pos).astype(np.uint32) << 16
                parts.append(raw.view(np.float32))
                pos += 2 * n
            else:
                parts.append(np.frombuffer(blob, "<f4", n, pos).astype(np.float32))
                pos += 4 * n
        if pos != len(blob):
            raise ValueError(f"{path}: {len(blob) - pos} trailing bytes")
        r = cls(0, ctx)
        r.set_params(np.concatenate(parts))
        return r

    # ---- data --------------------------------------------------------------
    def make_frames(self, frames: int, nfft: int = 1024, snr_db=(0.0, 40.0), seed: int = 0,
                    frame0: int = 0, truth: bool = False) -> dict:
        """Single-tone Hann frames made on the GPU -> dict of CUDA tensors:
        feat [F,10], target [F,2], parabolic [F,2] (bin, offset), valid [F]
        (int32 0/1) and, with truth=True, truth [F,2] (cycles/sample, SNR dB)."""
        import torch
        dev = torch.device("cuda", self.ctx.device)
        d = {"feat": torch.empty((frames, N_IN), dtype=torch.float32, device=dev),
             "target": torch.empty((frames, 2), dtype=torch.float32, device=dev),
             "parabolic": torch.empty((frames, 2), dtype=torch.float32, device=dev),
             "valid": torch.empty(frames, dtype=torch.int32, device=dev)}
        if truth:
            d["truth"] = torch.empty((frames, 2), dtype=torch.float32, device=dev)
        self.ctx.bind_stream()
        self.ctx.check(lib.spx_mlp_make_frames(
            self.ctx.h, int(seed), int(frame0), int(frames), int(nfft), float(snr_db[0]),
            float(snr_db[1]), _ptr(d["feat"]), _ptr(d["target"]), _ptr(d["parabolic"]),
            _ptr(d["valid"]), _ptr(d.get("truth"))))
        d["nfft"] = nfft
        return d

    # ---- network -----------------------------------------------------------
    def forward(self, x):
        import torch
        _check_rows(x, N_IN, "x")
        y = torch.empty((x.shape[0], N_OUT), dtype=torch.float32, device=x.device)
        self.ctx.bind_stream()
        self.ctx.check(lib.spx_mlp_forward(self.ctx.h, self.h, _ptr(x), x.shape[0], _ptr(y)))
        return y

    def gradients(self, x, t, mask=None):
        """-> (gradient [N_PARAMS] CUDA tensor, loss CUDA scalar tensor)."""
        import torch
        _check_rows(x, N_IN, "x")
        _check_rows(t, N_OUT, "t")
        g = torch.empty(N_PARAMS, dtype=torch.float32, device=x.device)
        loss = torch.zeros(1, dtype=torch.float32, device=x.device)
        self.ctx.bind_stream()
        self.ctx.check(lib.spx_mlp_gradients(self.ctx.h, self.h, _ptr(x), _ptr(t), _ptr(mask),
                                             x.shape[0], _ptr(g), _ptr(loss)))
        return g, loss

    def train_step(self, x, t, lr: float, mask=None):
        import torch
        _check_rows(x, N_IN, "x")
        _check_rows(t, N_OUT, "t")
        loss = torch.zeros(1, dtype=torch.float32, device=x.device)
        self.ctx.bind_stream()
        self.ctx.check(lib.spx_mlp_train_step(self.ctx.h, self.h, _ptr(x), _ptr(t), _ptr(mask),
                                              x.shape[0], float(lr), _ptr(loss)))
        return loss

    def train(self, data: dict, epochs: int = 20, batch: int = 4096, lr_max: float = 3e-3,
              lr_min: float = 1e-5, seed: int = 0) -> np.ndarray:
        """Minibatch Adam over data from make_frames (row count a power of
        two); returns the mean loss of every epoch."""
        import torch
        rows = data["feat"].shape[0]
        losses = torch.zeros(max(epochs, 1), dtype=torch.float32, device=data["feat"].device)
        self.ctx.bind_stream()
        self.ctx.check(lib.spx_mlp_train(self.ctx.h, self.h, _ptr(data["feat"]), _ptr(data["target"]),
                                         _ptr(data["valid"]), rows, int(batch), int(epochs),
                                         float(lr_max), float(lr_min), int(seed), _ptr(losses)))
        return losses[:epochs].cpu().numpy()

    def refine(self, spec, peaks, counts, n_point: int, sample_rate: float):
        """Rewrites freq_offset / refined_frequency of peaks ([beams, K, 8]
        int32 MaxValue words from topk/all_maxima, in place) from the complex
        spectrum spec [beams, nfft]; returns (amplitude [beams, K] float32,
        used [beams, K] int32: 1 where the network's estimate was kept)."""
        import torch
        beams, nfft = spec.reshape(-1, spec.shape[-1]).shape
        k = peaks.shape[1]
        amp = torch.zeros((beams, k), dtype=torch.float32, device=spec.device)
        used = torch.zeros((beams, k), dtype=torch.int32, device=spec.device)
        self.ctx.bind_stream()
        self.ctx.check(lib.spx_mlp_refine(self.ctx.h, self.h, _ptr(spec), beams, int(n_point), nfft,
                                          float(sample_rate), k, _ptr(peaks), _ptr(counts),
                                          _ptr(amp), _ptr(used)))
        return amp, used

    def fft_peaks(self, x, nfft: int, window: int, k: int, sample_rate: float = 1.0,
                  refine: int = 1, search_start: int = 0, search_end: int = 0, thresh_sigma: float = 0.0):
        """The top-K search of spx_fft_peaks on samples x [beams, n_point]
        complex64 with this network's refinement of every peak (one launch
        where the beam's spectrum fits one CTA): returns (peaks [beams, K, 8]
        int32 MaxValue words, counts [beams], amplitude [beams, K], used
        [beams, K]), the bits of fft_peaks + refine."""
        import torch
        from . import PEAK_TOPK, _require_cuda
        _require_cuda(x, torch.complex64, "x")
        x2 = x.reshape(-1, x.shape[-1])
        beams, n_point = x2.shape
        out = torch.zeros((beams, k, 8), dtype=torch.int32, device=x.device)
        counts = torch.zeros(beams, dtype=torch.int32, device=x.device)
        amp = torch.zeros((beams, k), dtype=torch.float32, device=x.device)
        used = torch.zeros((beams, k), dtype=torch.int32, device=x.device)
        p = _capi.peak_params(PEAK_TOPK, search_start, search_end, 0, k, refine, sample_rate, thresh_sigma)
        self.ctx.bind_stream()
        self.ctx.check(lib.spx_fft_peaks_mlp(self.ctx.h, self.h, _ptr(x2), beams, n_point, int(nfft), int(window),
                                             C.byref(p), _ptr(out), _ptr(counts), _ptr(amp), _ptr(used)))
        return out, counts, amp, used


def _check_rows(t, width, name):
    import torch
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()
            and t.dim() == 2 and t.shape[1] == width):
        raise ValueError(f"{name} must be a contiguous CUDA float32 tensor [rows, {width}]")
