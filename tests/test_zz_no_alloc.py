"""spx_all_maxima_noalloc: the all-maxima search for callers that must not
allocate device memory while they run (real-time loops that reserve their
memory at start-up, hosts that own all device memory through their own pool).

Called through the C ABI (ctypes) and checked against spx_all_maxima on the
same inputs, bit-exact (the test suite's tolerance for peak lists: every
field exact except phase within 1e-4 degree), on two calls in a row with
different shapes, so contents the fixed scratch array keeps from the previous
call cannot leak into the next.  This file is collected last on purpose; it
passes alone in a fresh process and after the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EXACT = ["index", "real", "imag", "magnitude", "freq_offset", "refined_frequency", "pad"]


def _spectrum(beams, nfft, seed):
    rng = np.random.default_rng(seed)
    z = (rng.standard_normal((beams, nfft)) + 1j * rng.standard_normal((beams, nfft))).astype(np.complex64)
    z[:, 100] += 500  # a strong line
    return z


def _outputs(z_dev, beams, cap):
    import torch
    out = torch.full((beams, cap, 8), -1, dtype=torch.int32, device=z_dev.device)
    counts = torch.full((beams,), -1, dtype=torch.int32, device=z_dev.device)
    return out, counts


def _run(spx, lib_fn, ctx, z_dev, mag_dev, beams, nfft, params, cap, bufs=None):
    out, counts = bufs if bufs is not None else _outputs(z_dev, beams, cap)
    ctx.bind_stream()
    st = lib_fn(ctx.h, C.c_void_p(mag_dev.data_ptr()) if mag_dev is not None else None,
                C.c_void_p(z_dev.data_ptr()), beams, nfft, C.byref(params),
                C.c_void_p(out.data_ptr()), C.c_void_p(counts.data_ptr()))
    ctx.check(st)
    return out, counts


def test_noalloc_matches_all_maxima_two_calls(spx, cuda):
    """The expected lists come from spx_all_maxima on the default context; the
    calls under test run on a context of their own, created here, whose
    grow-on-demand scratch no call has touched: a no-allocation call routed
    through that scratch would make it non-zero."""
    import torch
    ctx = spx.default_context()
    cases = [
        # beams, nfft, start, end, max_per_beam, refine, with_mag
        (4, 131072, 0, 0, 100000, spx.REFINE_PARABOLIC, True),   # 32 look-back tiles per beam
        (3, 16384, 7, 9000, 500, spx.REFINE_NONE, False),        # capacity-truncated
    ]
    data = []
    for i, (beams, nfft, s, e, mpb, refine, with_mag) in enumerate(cases):
        z = torch.from_numpy(_spectrum(beams, nfft, 40 + i)).to(cuda)
        mag = spx.magnitude(z) if with_mag else None
        p = spx.peak_params(spx.PEAK_ALL, s, e, 0, mpb, refine, 2048.0, 0.0)
        cap = spx._capi.all_maxima_capacity(nfft, s, e, mpb)[2]
        ref = _run(spx, spx.lib.spx_all_maxima, ctx, z, mag, beams, nfft, p, cap)
        data.append((z, mag, beams, nfft, p, cap, ref))
    torch.cuda.synchronize()

    # output buffers first, so that nothing but the call under test could allocate below
    bufs = [_outputs(d[0], d[2], d[5]) for d in data]
    fresh = spx.Context(cuda.index or 0)
    assert spx.lib.spx_scratch_bytes(fresh.h) == 0
    # set-up call: resolves the fixed array's address on this device and loads
    # the kernel's module (the first call on a device may allocate doing so)
    z, mag, beams, nfft, p, cap, _ = data[0]
    _run(spx, spx.lib.spx_all_maxima_noalloc, fresh, z, mag, beams, nfft, p, cap, bufs[0])
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]

    for (z, mag, beams, nfft, p, cap, (ref_out, ref_counts)), buf in zip(data, bufs):
        out, counts = _run(spx, spx.lib.spx_all_maxima_noalloc, fresh, z, mag, beams, nfft, p, cap, buf)
        torch.cuda.synchronize()
        rc = ref_counts.cpu().numpy()
        np.testing.assert_array_equal(counts.cpu().numpy(), rc)
        got = spx.maxvalues_to_numpy(out)
        ref = spx.maxvalues_to_numpy(ref_out)
        for b in range(beams):
            n = min(int(rc[b]), cap)
            for f in EXACT:
                np.testing.assert_array_equal(got[b, :n][f], ref[b, :n][f], err_msg=f)
            np.testing.assert_allclose(got[b, :n]["phase"], ref[b, :n]["phase"], atol=1e-4, rtol=0)
            assert n > 0

    torch.cuda.synchronize()
    assert spx.lib.spx_scratch_bytes(fresh.h) == 0, "the no-allocation entry point grew the context's scratch"
    assert torch.cuda.mem_get_info()[0] == free_before, "the no-allocation entry point allocated device memory"
    fresh.synchronize()  # no bounded device wait expired
    fresh.close()
    ctx.synchronize()


def test_noalloc_rejects_what_it_cannot_serve(spx, cuda):
    import torch
    ctx = spx.default_context()
    z = torch.zeros((1, 4096), dtype=torch.complex64, device=cuda)
    out = torch.empty((1, 2047, 8), dtype=torch.int32, device=cuda)
    counts = torch.empty(1, dtype=torch.int32, device=cuda)
    ctx.bind_stream()
    # a noise threshold needs per-beam histogram scratch
    p = spx.peak_params(spx.PEAK_ALL, 0, 0, 0, 1000, 0, 1.0, 6.0)
    st = spx.lib.spx_all_maxima_noalloc(ctx.h, None, C.c_void_p(z.data_ptr()), 1, 4096, C.byref(p),
                                        C.c_void_p(out.data_ptr()), C.c_void_p(counts.data_ptr()))
    assert st == spx._capi.SPX_ERR_INVALID_ARG
    assert b"thresh_sigma" in spx.lib.spx_last_error(ctx.h)
    # more look-back tiles than the fixed array holds (beams * ceil(span / 2048) > 32768)
    p = spx.peak_params(spx.PEAK_ALL, 0, 0, 0, 1000, 0, 1.0, 0.0)
    st = spx.lib.spx_all_maxima_noalloc(ctx.h, None, C.c_void_p(z.data_ptr()), 40000, 4096, C.byref(p),
                                        C.c_void_p(out.data_ptr()), C.c_void_p(counts.data_ptr()))
    assert st == spx._capi.SPX_ERR_INVALID_ARG
    assert b"exceeds the fixed scratch limit" in spx.lib.spx_last_error(ctx.h)
