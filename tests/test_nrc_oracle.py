"""FP64 radiance-cache oracle on the CPU: finite-difference gradient check,
Adam against a direct restatement, and the input encoding."""
import numpy as np

import oracle as O


def rand_net(seed=0, scale=1.0):
    r = np.random.default_rng(seed)
    dims = O.MLP_DIMS
    parts = [(r.uniform(-1, 1, dims[l] * dims[l + 1]) * np.sqrt(6.0 / dims[l]) * scale) for l in range(6)]
    return np.concatenate(parts).astype(np.float32)


def test_finite_difference_gradient_fp64():
    r = np.random.default_rng(1)
    w = rand_net(1)
    x = r.uniform(-1, 1, (8, 96)).astype(np.float32)
    t = r.uniform(0, 1, (8, 3)).astype(np.float32)
    y0, _, _ = O.mlp_forward_backward(w, x, None, emulate_bf16=False)
    den = y0 ** 2 + 0.01  # the training loss holds its denominator constant
    _, loss, dw = O.mlp_forward_backward(w, x, t, emulate_bf16=False, fixed_den=den)
    assert loss > 0
    idx = r.choice(len(w), 40, replace=False)
    # central differences on the weights (float32 storage: use a relative step)
    for i in idx:
        h = 1e-3 * max(1e-2, abs(float(w[i])))
        wp, wm = w.astype(np.float64).copy(), w.astype(np.float64).copy()
        wp[i] += h
        wm[i] -= h
        # the oracle reads float32 weights: perturb in float64 and check the
        # derivative of the loss through a float32 round trip of the step
        wp32, wm32 = wp.astype(np.float32), wm.astype(np.float32)
        hh = (float(wp32[i]) - float(wm32[i])) / 2
        if hh == 0:
            continue
        lp = O.mlp_forward_backward(wp32, x, t, emulate_bf16=False, grad=False, fixed_den=den)[1]
        lm = O.mlp_forward_backward(wm32, x, t, emulate_bf16=False, grad=False, fixed_den=den)[1]
        fd = (lp - lm) / (2 * hh)
        assert abs(fd - dw[i]) <= 1e-5 * max(1.0, abs(dw[i])) + 1e-7, (i, fd, dw[i])


def test_adam_matches_restatement():
    r = np.random.default_rng(2)
    n = 1000
    w = r.normal(size=n)
    m = np.zeros(n)
    v = np.zeros(n)
    w0 = w.copy()
    g1, g2 = r.normal(size=n), r.normal(size=n)
    O.adam_step(w, m, v, g1, 1, 1e-2)
    O.adam_step(w, m, v, g2, 2, 1e-2)
    mm = 0.1 * g1
    vv = 0.01 * g1 * g1
    ww = w0 - 1e-2 * (mm / 0.1) / (np.sqrt(vv / 0.01) + 1e-8)
    mm = 0.9 * mm + 0.1 * g2
    vv = 0.99 * vv + 0.01 * g2 * g2
    ww = ww - 1e-2 * (mm / (1 - 0.81)) / (np.sqrt(vv / (1 - 0.99 ** 2)) + 1e-8)
    assert np.allclose(w, ww, rtol=1e-12, atol=1e-14)


def test_encoding_layout():
    f = O.nrc_encode((0.5, 0.25, 1.0), (0, 0, 1), (0, 1, 0), 0.3, (0.1, 0.2, 0.3), (0, 0, 0), (1, 1, 1))
    assert f.shape == (96,)
    # x = 0.5: sin(pi/2) = 1, cos(pi/2) = 0 for band 0
    assert abs(f[0] - 1.0) < 1e-6 and abs(f[1]) < 1e-6
    # y = 0.25, band 1: sin(pi/2) = 1
    assert abs(f[24 + 2] - 1.0) < 1e-6
    assert np.allclose(f[72:82], [0, 0, 1, 0, 1, 0, 0.3, 0.1, 0.2, 0.3])
    assert np.all(f[82:] == 0)
