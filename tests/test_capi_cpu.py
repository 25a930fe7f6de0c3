"""CPU-only checks of the C ABI: the library loads, exports every symbol that
include/spx.h declares, and its host-only helpers follow the reference's
size rules.  No kernel is launched."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared_symbols():
    text = (ROOT / "include" / "spx.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(spx_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()  # no-op when the library is up to date
    from spectrum_gb300 import _capi
    return _capi.lib


def test_every_declared_symbol_is_exported_and_bound(lib):
    from spectrum_gb300 import _capi
    names = _declared_symbols()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), f"{n} declared in spx.h but not exported"
        assert n in _capi.PROTOTYPES, f"{n} has no ctypes prototype"
    assert set(_capi.PROTOTYPES) == set(names)


def test_abi_version_and_status_strings(lib):
    assert lib.spx_abi_version() == 1
    assert lib.spx_status_string(0) == b"SPX_OK"
    assert lib.spx_status_string(5) == b"SPX_ERR_TIMEOUT"


@pytest.mark.parametrize("n,expect", [(0, 1), (1, 1), (1000, 1024), (1024, 1024), (65537, 131072)])
def test_next_pow2(lib, n, expect):
    assert lib.spx_next_pow2(n) == expect


def test_next_smooth23_matches_oracle(lib):
    from oracle import spectrum_oracle as orc
    for n in list(range(1, 3000)) + [99999, 100000, 98305, 59049, 1 << 20]:
        assert lib.spx_next_smooth23(n) == orc.next_smooth23(n), n


def test_fft_size_support(lib):
    """2^a 3^b sizes by the Stockham plans, 2^19 .. 2^21 by the three-launch
    transform, 2^a 3^b sizes above 2^21 up to 2^28 that split into two
    factors <= 16384 by the four-step transform, every other length from 2
    to 2^27 by Bluestein's transform."""
    for n in (2, 3, 5, 7, 8, 1000, 1009, 4096, 13122, 59049, 104976, 131072, 262144, 524289, 3 << 18,
              1 << 19, (1 << 20) - 1, 1 << 20, (1 << 20) + 1, 1 << 21, 3 << 20, 1 << 22, 3 << 21, 1 << 24,
              3 ** 14, 3 ** 17, 1 << 27, (1 << 27) - 1, 1 << 28, (1 << 14) * 3 ** 8):
        assert lib.spx_fft_size_supported(n) == 1, n
    # too long for Bluestein's transform (non-smooth, > 2^27), beyond 2^28,
    # or 3-smooth beyond 2^28 (3^18); 3^17 has no split into two factors
    # <= 16384 and runs Bluestein's transform
    for n in (0, 1, (1 << 27) + 1, (1 << 28) + 1, 1 << 29, 3 ** 18, 0xFFFFFFFF):
        assert lib.spx_fft_size_supported(n) == 0, n


@pytest.mark.parametrize("nfft,start,end,maxpb", [
    (1024, 0, 0, 1000), (1024, 5, 2000, 10), (4096, 3000, 100, 1000), (131072, 0, 0, 1000), (8, 1, 2, 5)])
def test_all_maxima_capacity_matches_reference_rule(lib, nfft, start, end, maxpb):
    from oracle import spectrum_oracle as orc
    from spectrum_gb300 import _capi
    assert _capi.all_maxima_capacity(nfft, start, end, maxpb) == orc.all_maxima_capacity(nfft, start, end, maxpb)


def test_noise_threshold_factor(lib):
    from oracle import spectrum_oracle as orc
    for s in (0.0, 3.0, 6.0, 10.5):
        assert lib.spx_noise_threshold_factor(s) == float(orc.noise_threshold_factor(s))
    assert abs(lib.spx_noise_threshold_factor(6.0) - 4.4024) < 1e-3


def test_create_without_gpu_reports_no_device(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert lib.spx_create(0, C.byref(h)) == 6  # SPX_ERR_NO_DEVICE
    assert not h.value


def test_null_context_is_invalid_argument(lib):
    assert lib.spx_fft(None, None, 1, 1, 1, 0, 0, 1.0, None) == 1
    assert lib.spx_destroy(None) == 0
    assert lib.spx_last_error(None) == b""
    assert lib.spx_scratch_bytes(None) == 0


def test_every_entry_point_rejects_null_handles(lib):
    """Every call whose first argument is a context, batch or MLP handle returns
    SPX_ERR_INVALID_ARG for null handles and zero sizes, before it touches a
    device; the destroy calls accept null, like free()."""
    from spectrum_gb300 import _capi
    destroy = {"spx_destroy", "spx_batch_destroy", "spx_mlp_destroy"}
    checked = 0
    for name, (res, args) in _capi.PROTOTYPES.items():
        if res is not C.c_int or not args or args[0] is not C.c_void_p:
            continue
        vals = [0.0 if a is C.c_float else 0 if a in (C.c_uint32, C.c_int, C.c_uint64) else None
                for a in args]
        assert getattr(lib, name)(*vals) == (0 if name in destroy else 1), name
        checked += 1
    assert checked >= 30


@pytest.mark.parametrize("call", ["fft", "ifft", "fft_r2c", "topk", "all_maxima", "fft_peaks",
                                  "host_dtype", "host_strided"])
def test_python_wrappers_reject_bad_tensors_before_any_device_work(lib, call):
    """The Python mirror checks device, dtype and layout first, like the
    reference's std::invalid_argument checks, and raises ValueError."""
    import torch

    import spectrum_gb300 as spx
    x = torch.zeros((2, 64), dtype=torch.complex64)
    calls = {
        "fft": lambda: spx.fft(x, 64),
        "ifft": lambda: spx.ifft(x),
        "fft_r2c": lambda: spx.fft_r2c(torch.zeros((2, 64)), 64),
        "topk": lambda: spx.topk(x, 5),
        "all_maxima": lambda: spx.all_maxima(x),
        "fft_peaks": lambda: spx.fft_peaks(x, 64),
        "host_dtype": lambda: spx.fft_peaks_host(torch.zeros((2, 64)), 64),
        "host_strided": lambda: spx.fft_peaks_host(x.t(), 64),
    }
    with pytest.raises(ValueError):
        calls[call]()
