"""GPU tests of uneven batches (spx_batch_*): the single launch, the per-size
launches and the CUDA-graph replay give bit-identical top-K lists; without a
window they also equal the oracle's top-K on spx_fft's spectrum of every beam
(same FFT code, same plans)."""
import numpy as np
import pytest

from oracle import spectrum_oracle as orc

pytestmark = pytest.mark.gpu

EXACT = ["index", "real", "imag", "magnitude", "freq_offset", "refined_frequency", "pad"]


def _uneven(beams, lo, hi, seed, extra=()):
    from spectrum_gb300 import synth
    rng = np.random.default_rng(seed)
    lengths = list(rng.integers(lo, hi, beams)) + list(extra)
    bs = synth.make_beams(lengths, tones=(1, 8), snr_db=(0.0, 40.0), seed=seed)
    rows = synth.synth_numpy(bs)
    flat = np.concatenate([rows[i, :n] for i, n in enumerate(bs.lengths)])
    return np.asarray(bs.lengths, np.uint32), flat.astype(np.complex64)


def _same(a, b):
    for f in EXACT + ["phase"]:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)


@pytest.mark.parametrize("window", [0, 1])
def test_batch_single_launch_equals_per_size_and_graph(spx, cuda, window):
    import torch
    from spectrum_gb300.batch import Batch
    # sizes cover cluster sizes 1, 2, 3, 4, 6, 8 and 9 (59049 = 3^10)
    n_points, x = _uneven(40, 1000, 20000, 5, extra=(33000, 52000, 59049, 70000, 99000, 100000))
    xd = torch.from_numpy(x).to(cuda)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        b = Batch(n_points, window=window, k=8, sample_rate=1.0)
        o1, c1 = [t.clone() for t in b.run(xd)]
        o2, c2 = [t.clone() for t in b.run_per_size(xd)]
        b.capture(xd, stream=s)
        o3, c3 = [t.clone() for t in b.replay(stream=s)]
    torch.cuda.synchronize()
    for o, c in ((o2, c2), (o3, c3)):
        np.testing.assert_array_equal(c.cpu().numpy(), c1.cpu().numpy())
        _same(spx.maxvalues_to_numpy(o), spx.maxvalues_to_numpy(o1))
    assert (c1.cpu().numpy() == 8).all()


def test_batch_matches_oracle_without_window(spx, cuda):
    import torch
    from spectrum_gb300.batch import Batch
    n_points, x = _uneven(12, 1000, 30000, 9, extra=(65536, 98000))
    xd = torch.from_numpy(x).to(cuda)
    b = Batch(n_points, window=0, k=8, sample_rate=2.0)
    out, counts = b.run(xd)
    got = spx.maxvalues_to_numpy(out)
    counts = counts.cpu().numpy()
    off = 0
    for i, n in enumerate(n_points):
        nfft = spx.next_smooth23(int(n))
        spec = spx.fft(xd[off:off + n].reshape(1, -1), nfft).cpu().numpy()
        ref, rc = orc.topk(None, spec, nfft, 2.0, 8)
        assert counts[i] == rc[0]
        for f in EXACT:
            np.testing.assert_array_equal(got[i, : rc[0]][f], ref[0, : rc[0]][f], err_msg=f"beam {i} {f}")
        off += int(n)


def test_batch_autotune_keeps_results_and_plan_cache_round_trips(spx, cuda, tmp_path):
    """The autotuner picks a local FFT size per distinct nfft by timing; any
    choice gives the same lists bit for bit when the plain path uses the same
    plan (the batch's plans are the context's).  A saved plan file loads back
    into a new batch with the same plans and results."""
    import torch
    from spectrum_gb300.batch import Batch
    n_points, x = _uneven(16, 1000, 40000, 13, extra=(80000, 93312))
    xd = torch.from_numpy(x).to(cuda)
    ctx = spx.Context(0)
    b = Batch(n_points, window=1, k=4, ctx=ctx)
    o1, c1 = [t.clone() for t in b.run(xd)]
    tuned, changed = b.autotune(xd)
    assert tuned >= 2 and 0 <= changed <= tuned
    o2, c2 = [t.clone() for t in b.run(xd)]
    np.testing.assert_array_equal(c1.cpu().numpy(), c2.cpu().numpy())
    # every beam equals spx_fft_peaks on the same context (same plans)
    g2 = spx.maxvalues_to_numpy(o2)
    off = 0
    for i, n in enumerate(n_points):
        o, c = spx.fft_peaks(xd[off:off + int(n)].reshape(1, -1), b.nffts[i], 1, spx.PEAK_TOPK, sample_rate=1.0,
                             max_per_beam=4, refine=spx.REFINE_PARABOLIC, ctx=ctx)
        _same(spx.maxvalues_to_numpy(o)[0, :int(c[0])], g2[i, :int(c[0])])
        off += int(n)
    # force a different plan for 93312 = 6 x 15552 = 8 x 11664 and a larger
    # cluster than the largest C, and round-trip the cache
    b.set_local_size(93312, 11664)
    assert b.local_size(93312) == 11664
    b.set_cluster(16)  # at least the largest C, whatever the autotuner chose
    assert b.cluster == 16
    path = tmp_path / "plans.json"
    b.save_plans(path)
    assert '"93312": 11664' in path.read_text() and '"cluster": 16' in path.read_text()
    b2 = Batch(n_points, window=1, k=4, ctx=spx.Context(0))
    assert b2.load_plans(path) == len(b.plans)
    assert b2.plans == b.plans and b2.cluster == 16
    o3, c3 = [t.clone() for t in b.run(xd)]
    o4, c4 = [t.clone() for t in b2.run(xd)]
    np.testing.assert_array_equal(c3.cpu().numpy(), c4.cpu().numpy())
    _same(spx.maxvalues_to_numpy(o3), spx.maxvalues_to_numpy(o4))
    with pytest.raises(ValueError):
        b.set_local_size(93312, 1000)   # not C x M with C in the batch's cluster sizes
    with pytest.raises(ValueError):
        b.set_cluster(2)                # smaller than the >= 8 CTAs of 93312 = 8 x 11664
    with pytest.raises(ValueError):
        b.set_cluster(17)               # beyond 16
    with pytest.raises(spx._capi.SpxError):
        b.tune(32)                      # batches run 16 points per thread


@pytest.mark.parametrize("n_point,nfft", [(500000, 0), (4096, 1 << 20), (4096, 1 << 22)])
def test_batch_rejects_three_launch_sizes(spx, cuda, n_point, nfft):
    """A beam whose transform is 2^19 points or more (the next 3-smooth size
    of 500000 is 2^19, or an explicit nfft of 2^20 or of 2^22, a four-step
    transform) is not a cluster of the batch kernel: creation fails with
    SPX_ERR_UNSUPPORTED, nothing is launched, and the context keeps working."""
    from spectrum_gb300 import _capi
    from spectrum_gb300.batch import Batch
    n_points = [1000, n_point]
    nffts = None if nfft == 0 else [0, nfft]
    with pytest.raises(_capi.SpxError) as ei:
        Batch(n_points, nffts=nffts, window=spx.WINDOW_HANN, k=4, sample_rate=1.0)
    assert ei.value.status == _capi.SPX_ERR_UNSUPPORTED
    assert "2^19 points and more" in str(ei.value)
    lengths, flat = _uneven(6, 1000, 5000, seed=11)
    b = Batch(lengths, window=spx.WINDOW_HANN, k=4, sample_rate=1.0)
    import torch
    out, counts = b.run(torch.from_numpy(flat).to(cuda))
    assert int(counts.min()) >= 1


@pytest.mark.parametrize("cluster", [0, 9, 10, 12, 16])
def test_batch_cluster_size_keeps_results(spx, cuda, cluster):
    """Any cluster size of the single launch from the largest C up to 16
    packs the same beams differently and gives the same lists bit for bit."""
    import torch
    from spectrum_gb300.batch import Batch
    n_points, x = _uneven(24, 1000, 60000, 29, extra=(59049, 80000))
    xd = torch.from_numpy(x).to(cuda)
    b = Batch(n_points, window=spx.WINDOW_HANN, k=8, sample_rate=1.0)
    o1, c1 = [t.clone() for t in b.run(xd)]
    b.set_cluster(cluster)
    assert b.cluster == (9 if cluster == 0 else cluster)  # 59049 = 9 x 6561
    o2, c2 = [t.clone() for t in b.run(xd)]
    np.testing.assert_array_equal(c1.cpu().numpy(), c2.cpu().numpy())
    _same(spx.maxvalues_to_numpy(o1), spx.maxvalues_to_numpy(o2))
