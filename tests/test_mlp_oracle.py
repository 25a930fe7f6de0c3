"""CPU checks of the learned-refinement oracle: its backward pass against
central finite differences (FP64, weights unrounded so the loss is smooth),
BF16 rounding, and the label/feature definitions on a noiseless tone."""
import numpy as np

from oracle import mlp_oracle as mo


def test_bf16_round_known_values():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -2.5, 0.0], np.float32)
    # 1 + 2^-8 is a tie -> even (1.0); 1 + 3*2^-8 is a tie -> even (1 + 2^-6)
    np.testing.assert_array_equal(mo.bf16_round(x),
                                  np.array([1.0, 1.0, 1.0 + 2 ** -7, 1.0 + 2 ** -6, -2.5, 0.0], np.float32))


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = (rng.standard_normal(mo.N_PARAMS) * 0.3).astype(np.float64)
    x = rng.standard_normal((40, mo.N_IN))
    t = rng.standard_normal((40, mo.N_OUT))
    mask = (rng.uniform(size=40) > 0.3).astype(np.uint32)
    _, g = mo.loss_and_grad(p, x, t, mask, round_weights=False)
    idx = rng.choice(mo.N_PARAMS, 200, replace=False)
    h = 1e-5
    for i in idx:
        e = np.zeros(mo.N_PARAMS)
        e[i] = h
        lp, _ = mo.loss_and_grad(p + e, x, t, mask, round_weights=False)
        lm, _ = mo.loss_and_grad(p - e, x, t, mask, round_weights=False)
        assert abs((lp - lm) / (2 * h) - g[i]) < 1e-7 + 1e-5 * abs(g[i]), i


def test_oracle_adam_first_step_is_signed_lr():
    g = np.array([1e-3, -2.0, 5.0])
    p, m, v = mo.adam_step(np.zeros(3), np.zeros(3), np.zeros(3), g, 0.01, 1)
    np.testing.assert_allclose(p, -0.01 * np.sign(g), rtol=1e-4)


def test_labels_of_a_noiseless_tone():
    """A pure tone between bins: the 16x zero-padded judge finds its offset
    to ~1e-4 bin, the parabola on the coarse Hann spectrum is biased, and the
    main-lobe phase features are ~0 after the window's linear phase is removed."""
    n = 1024
    for off in (-0.41, -0.2, 0.0, 0.13, 0.37):
        k = 200
        f = (k + off) / n
        x = np.exp(2j * np.pi * f * np.arange(n)) * mo.hann(n)
        X = np.fft.fft(x)
        X16 = np.fft.fft(x, 16 * n)
        o, la = mo.fine_label(X16, k, X)
        assert abs(o - off) < 2e-4
        feat = mo.peak_features(X, k, n, n)
        assert np.all(np.abs(feat[6:9]) < 1e-6)
        a = np.abs(X[k - 1:k + 2])
        den = a[0] - 2 * a[1] + a[2]
        par = 0.5 * (a[0] - a[2]) / den
        if off != 0.0:
            assert abs(par - off) > 1e-3     # scalloping bias the network removes
        # amplitude: |X[k]| exp(la) = the window's coherent gain (sum of Hann = (n-1)/2)
        assert abs(np.abs(X[k]) * np.exp(la) - (n - 1) / 2) / ((n - 1) / 2) < 1e-4
