"""GPU checks of the learned sub-bin refinement (spx_mlp_*).

* forward, gradients and one Adam step of the hand-written kernels against
  the FP64 oracle (BF16-rounded weights on both sides);
* training frames and labels made on the GPU against the oracle's features
  and 16x zero-padded judge on noiseless tones;
* the trained network against the parabola it replaces: frequency RMS error
  at SNR 20 dB at least 3x lower, on the training frame size (nFFT 1024) and
  on the inference workload (4096 beams x 8192 samples);
* the fused inference kernel against the oracle on the same spectrum;
* save/load round trip and argument checks.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def learned(spx):
    from spectrum_gb300 import learned
    return learned


@pytest.fixture(scope="module")
def trained(learned, cuda):
    """The network trained as the learned-refinement workload specifies:
    2^20 single-tone Hann frames of 1024 samples, SNR U[0, 40] dB."""
    r = learned.MLPRefiner(seed=1)
    data = r.make_frames(1 << 20, nfft=1024, snr_db=(0.0, 40.0), seed=11)
    losses = r.train(data, epochs=20, batch=4096, lr_max=3e-3, lr_min=1e-5, seed=5)
    return r, losses, data


def _rand(rows, seed, cuda):
    import torch
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((rows, 10)).astype(np.float32)
    t = (rng.standard_normal((rows, 2)) * 0.3).astype(np.float32)
    m = (rng.uniform(size=rows) > 0.25).astype(np.int32)
    return x, t, m, torch.from_numpy(x).to(cuda), torch.from_numpy(t).to(cuda), torch.from_numpy(m).to(cuda)


def test_forward_matches_oracle(learned, cuda):
    r = learned.MLPRefiner(seed=3)
    x, _, _, xd, _, _ = _rand(3000, 1, cuda)
    got = r.forward(xd).cpu().numpy()
    ref, _ = mo.forward(r.params, x)
    np.testing.assert_allclose(got, ref, rtol=0, atol=2e-5 * np.abs(ref).max())


@pytest.mark.parametrize("rows,masked", [(1, False), (777, True), (5000, True), (4096, False)])
def test_gradients_match_oracle(learned, cuda, rows, masked):
    r = learned.MLPRefiner(seed=rows)
    x, t, m, xd, td, md = _rand(rows, rows + 1, cuda)
    g, loss = r.gradients(xd, td, md if masked else None)
    lref, gref = mo.loss_and_grad(r.params, x, t, m if masked else None)
    g = g.cpu().numpy()
    assert abs(float(loss.item()) - lref) <= 1e-5 * lref + 1e-12
    off = 0
    for shape in mo.SHAPES:
        n = int(np.prod(shape))
        a, b = g[off:off + n], gref[off:off + n]
        assert np.abs(a - b).max() <= 2e-5 * np.abs(b).max() + 1e-10, shape
        off += n


def test_adam_step_matches_oracle(learned, cuda):
    r = learned.MLPRefiner(seed=9)
    x, t, m, xd, td, md = _rand(2048, 4, cuda)
    p0 = r.params
    _, g = mo.loss_and_grad(p0, x, t, m)
    p1 = p0.astype(np.float64)
    mm = np.zeros_like(p1)
    vv = np.zeros_like(p1)
    for step in (1, 2):
        # second step: gradient at the new (BF16-rounded) weights
        if step == 2:
            _, g = mo.loss_and_grad(p1.astype(np.float32), x, t, m)
        p1, mm, vv = mo.adam_step(p1, mm, vv, g, 1e-3, step)
        r.train_step(xd, td, 1e-3, md)
    got = r.params
    # an update is lr * m/(sqrt(v)+eps): parameters whose gradient is ~0 can flip sign
    big = np.abs(g) > 1e-3 * np.abs(g).max()
    np.testing.assert_allclose(got[big], p1[big], rtol=0, atol=2e-5)
    np.testing.assert_allclose(got, p1, rtol=0, atol=2.1e-3)


def test_frames_and_labels_match_oracle(learned, cuda):
    """SNR 300 dB (noise 1e-15): features and labels are functions of the
    tone frequency alone (the random phase cancels), so the oracle rebuilds
    them from the returned truth."""
    r = learned.MLPRefiner(seed=0)
    n = 1024
    d = r.make_frames(64, nfft=n, snr_db=(300.0, 300.0), seed=3, truth=True)
    feat = d["feat"].cpu().numpy()
    tgt = d["target"].cpu().numpy()
    par = d["parabolic"].cpu().numpy()
    assert (d["valid"].cpu().numpy() == 1).all()
    truth = d["truth"].cpu().numpy()
    t = np.arange(n)
    for i in range(64):
        f = float(truth[i, 0])
        x = np.exp(2j * np.pi * f * t) * mo.hann(n)
        X = np.fft.fft(x)
        k = int(par[i, 0])
        assert abs(k - f * n) <= 0.5 + 1e-3
        fe = mo.peak_features(X, k, n, n)
        np.testing.assert_allclose(feat[i, :5], fe[:5], atol=2e-5)
        ok = fe[:5] > 1e-3          # phase of a near-zero bin is not defined
        dph = np.angle(np.exp(1j * (feat[i, 5:] - fe[5:])))
        assert np.all(np.abs(dph[ok]) < 1e-3), (i, dph)
        off, la = mo.fine_label(np.fft.fft(x, 16 * n), k, X)
        assert abs(tgt[i, 0] - off) < 1e-4
        assert abs(tgt[i, 1] - la) < 1e-4
        assert abs(tgt[i, 0] - (f * n - k)) < 5e-4      # the judge itself
        a = np.abs(X[k - 1:k + 2])
        assert abs(par[i, 1] - 0.5 * (a[0] - a[2]) / (a[0] - 2 * a[1] + a[2])) < 1e-4


def test_gradients_and_training_are_reproducible(learned, cuda):
    """The weight gradients are summed per chunk of rows, then over chunks in
    a fixed order (no atomics): the same inputs give the same bits, and two
    trainings from the same seed on the same frames end with identical
    weights."""
    r = learned.MLPRefiner(seed=21)
    _, _, _, xd, td, md = _rand(5000, 22, cuda)
    g1, _ = r.gradients(xd, td, md)
    g2, _ = r.gradients(xd, td, md)
    assert np.array_equal(g1.cpu().numpy().view(np.uint32), g2.cpu().numpy().view(np.uint32))
    data = r.make_frames(1 << 16, nfft=1024, snr_db=(0.0, 40.0), seed=23)
    runs = []
    for _ in range(2):
        m = learned.MLPRefiner(seed=24)
        m.train(data, epochs=2, batch=4096, lr_max=3e-3, lr_min=1e-5, seed=25)
        runs.append(m.params.view(np.uint32).copy())
        m.close()
    assert np.array_equal(runs[0], runs[1])


def test_training_reduces_loss(trained):
    _, losses, data = trained
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.05 * losses[0]
    assert float(data["valid"].float().mean().item()) > 0.999


def test_learned_beats_parabolic_at_20db_nfft1024(trained):
    """Frequency RMS error vs the true tone, held-out frames at SNR 20 dB."""
    r, _, _ = trained
    n = 1024
    d = r.make_frames(1 << 15, nfft=n, snr_db=(20.0, 20.0), seed=99, truth=True)
    valid = d["valid"].cpu().numpy() == 1
    k = d["parabolic"][:, 0].cpu().numpy()
    truth = d["truth"][:, 0].cpu().numpy().astype(np.float64) * n - k
    par = d["parabolic"][:, 1].cpu().numpy()
    y = r.forward(d["feat"]).cpu().numpy()
    use = np.abs(y[:, 0]) <= 0.5
    est = np.where(use, y[:, 0], par)
    rms_p = np.sqrt(np.mean((par - truth)[valid] ** 2))
    rms_m = np.sqrt(np.mean((est - truth)[valid] ** 2))
    print(f"nfft 1024 @20 dB: parabolic {rms_p:.5f} bins, learned {rms_m:.5f} bins, "
          f"gain {rms_p / rms_m:.2f}x, fallback {1 - use[valid].mean():.4f}")
    assert rms_p / rms_m >= 3.0


def test_learned_beats_parabolic_inference_workload(spx, trained, cuda):
    """4096 beams x 8192 samples, one tone each at SNR 20 dB: top-1 with the
    parabola, then the fused refinement kernel; frequency RMS error in bins
    against the planted tones (tones within 4 bins of the band edges left out)."""
    import torch
    from spectrum_gb300 import synth
    r, _, _ = trained
    bs = synth.workload_learned(seed=4)
    xd = synth.synth_torch(bs, device=cuda)
    n = 8192
    spec = spx.fft(xd, n, window=spx.WINDOW_HANN)
    out, counts = spx.topk(spec, 1, sample_rate=1.0, refine=spx.REFINE_PARABOLIC)
    par = spx.maxvalues_to_numpy(out)[:, 0].copy()
    amp, used = r.refine(spec, out, counts, n, 1.0)
    got = spx.maxvalues_to_numpy(out)[:, 0]
    used = used.cpu().numpy()[:, 0]
    f = np.array([fr[0] for fr in bs.freqs]) * n
    keep = (f > 4) & (f < n / 2 - 4) & (counts.cpu().numpy() == 1)
    ep = (par["index"] + par["freq_offset"].astype(np.float64)) - f
    em = (got["index"] + got["freq_offset"].astype(np.float64)) - f
    rms_p = np.sqrt(np.mean(ep[keep] ** 2))
    rms_m = np.sqrt(np.mean(em[keep] ** 2))
    print(f"4096 x 8192 @20 dB: parabolic {rms_p:.5f} bins, learned {rms_m:.5f} bins, "
          f"gain {rms_p / rms_m:.2f}x, network used on {used[keep].mean():.4f}")
    assert rms_p / rms_m >= 3.0
    # the refined frequency follows the reference's formula from the new offset
    u = used == 1
    np.testing.assert_array_equal(
        got["refined_frequency"][u],
        ((got["index"][u].astype(np.float32) + got["freq_offset"][u]) * np.float32(1.0 / n)).astype(np.float32))
    # where the network was not used the parabolic values stay
    nu = used == 0
    np.testing.assert_array_equal(got["freq_offset"][nu], par["freq_offset"][nu])
    # fused kernel vs the oracle network on the same spectrum (sample of beams)
    p = r.params
    sp = spec[:256].cpu().numpy()
    for b in range(256):
        if not keep[b]:
            continue
        k = int(par["index"][b])
        y, _ = mo.forward(p, mo.peak_features(sp[b], k, n, n)[None])
        if abs(y[0, 0]) < 0.499:
            assert used[b] == 1
            assert abs(got["freq_offset"][b] - y[0, 0]) < 1e-4
            assert abs(amp[b, 0].item() - par["magnitude"][b] * np.exp(y[0, 1])) < 1e-4 * par["magnitude"][b]


@pytest.mark.parametrize("beams,n,k,sigma,win", [
    (256, 8192, 1, 0.0, 1),    # the inference workload's shape, 2^21 points (one launch)
    (512, 8192, 1, 0.0, 1),    # 2^22 points: spectrum, search, refinement
    (16, 4096, 8, 0.0, 1),     # one launch, K = 8
    (8, 16384, 3, 3.0, 4),     # one launch, threshold, Blackman-Harris
    (12, 6561, 4, 0.0, 2),     # 3-smooth, one launch
    (8, 1024, 2, 0.0, 1),      # too small for the weights: spectrum, search, refinement
])
def test_fft_peaks_mlp_matches_the_three_steps(spx, trained, cuda, beams, n, k, sigma, win):
    """spx_fft_peaks_mlp (transform, top-K and the network on every peak in one
    launch where the spectrum and the weights fit one CTA) gives the records,
    amplitudes and used flags of spx_fft + spx_topk + spx_mlp_refine, bit for
    bit."""
    from spectrum_gb300 import synth
    r, _, _ = trained
    bs = synth.make_beams([n] * beams, tones=(1, 3), snr_db=(10.0, 30.0), seed=n + k)
    xd = synth.synth_torch(bs, device=cuda)
    out, counts, amp, used = r.fft_peaks(xd, n, win, k, sample_rate=2.0, thresh_sigma=sigma)
    spec = spx.fft(xd, n, window=win)
    o2, c2 = spx.topk(spec, k, sample_rate=2.0, refine=spx.REFINE_PARABOLIC, thresh_sigma=sigma)
    a2, u2 = r.refine(spec, o2, c2, n, 2.0)
    np.testing.assert_array_equal(counts.cpu().numpy(), c2.cpu().numpy())
    c = counts.cpu().numpy()
    g1, g2 = spx.maxvalues_to_numpy(out), spx.maxvalues_to_numpy(o2)
    a1, a2n, u1, u2n = amp.cpu().numpy(), a2.cpu().numpy(), used.cpu().numpy(), u2.cpu().numpy()
    for b in range(beams):
        m = int(c[b])
        for f in ("index", "real", "imag", "magnitude", "phase", "freq_offset", "refined_frequency"):
            np.testing.assert_array_equal(g1[b, :m][f], g2[b, :m][f], err_msg=f"beam {b} {f}")
        np.testing.assert_array_equal(a1[b, :m], a2n[b, :m])
        np.testing.assert_array_equal(u1[b, :m], u2n[b, :m])
    assert u1.sum() > 0  # the network was used somewhere


def test_save_load_round_trip(learned, trained, cuda, tmp_path):
    import torch
    r, _, _ = trained
    path = tmp_path / "refiner.spxmlp"
    r.save(path)
    r2 = learned.MLPRefiner.load(path)
    x = torch.randn((1000, 10), device=cuda)
    np.testing.assert_array_equal(r.forward(x).cpu().numpy(), r2.forward(x).cpu().numpy())
    p, p2 = r.params, r2.params
    np.testing.assert_array_equal(mo.bf16_round(p[:640]), p2[:640])
    np.testing.assert_array_equal(p[640:704], p2[640:704])
    blob = path.read_bytes()
    assert blob[:8] == b"SPXMLP1\n"
    with pytest.raises(ValueError):
        path.write_bytes(blob + b"\0")
        learned.MLPRefiner.load(path)


def test_argument_checks(learned, cuda):
    import torch
    r = learned.MLPRefiner(seed=0)
    with pytest.raises(ValueError):
        r.make_frames(4, nfft=1000)
    with pytest.raises(ValueError):
        r.make_frames(4, nfft=1024, snr_db=(30.0, 10.0))
    d = r.make_frames(12, nfft=256)
    with pytest.raises(ValueError):
        r.train(d, epochs=1, batch=4)          # 12 rows: not a power of two
    with pytest.raises(ValueError):
        r.forward(torch.zeros((3, 9), device=cuda))
