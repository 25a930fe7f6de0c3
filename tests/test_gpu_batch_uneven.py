"""The uneven-batch workload at full size: 1024 beams, n_point U[1000, 100000],
nFFT = next 2^a 3^b (58 distinct sizes), Hann window, top-8 strict local
maxima with parabolic refinement (synth.workload_uneven).

* Plain path: each beam alone through spx_fft_peaks (its own window table,
  its own per-size FFT plan and kernels) gives the batch's top-8 list bit for
  bit, every field, for all 1024 beams.  The batch evaluates the window per
  sample with the same function that fills the plain path's tables, and uses
  the same plans, so the spectra are the same bits.
* Oracle: on spx_fft's spectrum of one beam of every distinct nFFT plus
  random others (72 beams), orc.topk gives the batch's lists (indices,
  counts, every field; phase within 1e-4 degree).
* FP64: those beams' spectra against an FP64 FFT of the samples times the
  FP64 window: max |dX| <= 1e-6 of the beam's largest |X|, and the detected
  peaks' |X| within 1e-5 relative for peaks at >= 1e-2 of the beam's largest.
"""
import numpy as np
import pytest

from oracle import spectrum_oracle as orc

pytestmark = pytest.mark.gpu

EXACT = ["index", "real", "imag", "magnitude", "freq_offset", "refined_frequency", "pad"]


@pytest.fixture(scope="module")
def uneven(spx, cuda):
    import torch

    from spectrum_gb300 import synth
    from spectrum_gb300.batch import Batch
    bs = synth.workload_uneven(seed=2)
    x = synth.synth_torch(bs, device=cuda, packed=True)
    b = Batch(bs.lengths, window=spx.WINDOW_HANN, k=8, sample_rate=1.0)
    out, counts = [t.clone() for t in b.run(x)]
    torch.cuda.synchronize()
    offs = np.concatenate([[0], np.cumsum(bs.lengths)]).astype(np.int64)
    return bs, x, offs, spx.maxvalues_to_numpy(out), counts.cpu().numpy(), b


def test_uneven_workload_batch_equals_plain_path_every_beam(spx, cuda, uneven):
    bs, x, offs, got, counts, _ = uneven
    assert len(bs.lengths) == 1024
    nffts = [spx.next_smooth23(int(n)) for n in bs.lengths]
    assert len(set(nffts)) >= 50
    for i, n in enumerate(bs.lengths):
        beam = x[offs[i]:offs[i + 1]].reshape(1, -1)
        o, c = spx.fft_peaks(beam, nffts[i], spx.WINDOW_HANN, spx.PEAK_TOPK, sample_rate=1.0,
                             max_per_beam=8, refine=spx.REFINE_PARABOLIC)
        ref = spx.maxvalues_to_numpy(o)[0]
        rc = int(c.cpu()[0])
        assert counts[i] == rc, f"beam {i} (n_point {n}, nfft {nffts[i]})"
        for f in EXACT + ["phase"]:
            np.testing.assert_array_equal(got[i, :rc][f], ref[:rc][f], err_msg=f"beam {i} {f}")


def _sample_beams(nffts, seed=7, extra=14):
    first = {}
    for i, n in enumerate(nffts):
        first.setdefault(n, i)
    rng = np.random.default_rng(seed)
    rest = [i for i in rng.permutation(len(nffts)) if i not in first.values()][:extra]
    return sorted(list(first.values()) + rest)


def test_uneven_workload_batch_matches_oracle_and_fp64(spx, cuda, uneven):
    bs, x, offs, got, counts, _ = uneven
    nffts = [spx.next_smooth23(int(n)) for n in bs.lengths]
    beams = _sample_beams(nffts)
    assert len(beams) >= 64 and len({nffts[i] for i in beams}) == len(set(nffts))
    worst_abs, worst_peak = 0.0, 0.0
    for i in beams:
        n, nfft = int(bs.lengths[i]), nffts[i]
        beam = x[offs[i]:offs[i + 1]].reshape(1, -1)
        spec = spx.fft(beam, nfft, window=spx.WINDOW_HANN).cpu().numpy()
        ref, rc = orc.topk(None, spec, nfft, 1.0, 8)
        assert counts[i] == rc[0], f"beam {i}"
        for f in EXACT:
            np.testing.assert_array_equal(got[i, :rc[0]][f], ref[0, :rc[0]][f], err_msg=f"beam {i} {f}")
        np.testing.assert_allclose(got[i, :rc[0]]["phase"], ref[0, :rc[0]]["phase"], atol=1e-4, rtol=0)
        # FP64: the FP32 samples times the exact window, transformed in FP64
        t = np.arange(n)
        w = np.sin(np.pi * t / (n - 1)) ** 2
        x64 = beam.cpu().numpy()[0].astype(np.complex128) * w
        X = np.fft.fft(x64, nfft)
        peak = np.abs(X).max()
        worst_abs = max(worst_abs, float(np.abs(spec[0] - X).max() / peak))
        k = got[i, :rc[0]]["index"].astype(np.int64)
        mk = np.abs(X[k])
        strong = mk >= 1e-2 * peak
        if strong.any():
            rel = np.abs(got[i, :rc[0]]["magnitude"].astype(np.float64)[strong] - mk[strong]) / mk[strong]
            worst_peak = max(worst_peak, float(rel.max()))
    print(f"uneven workload, {len(beams)} beams: max |dX| / peak vs FP64 {worst_abs:.3e}; "
          f"peak |X| relative error vs FP64 {worst_peak:.3e}")
    assert worst_abs <= 1e-6
    assert worst_peak <= 1e-5
