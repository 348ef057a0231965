"""The numpy MLP restatement checks itself: analytic gradients against central differences.

It is the checker of the CUDA forward / backward / Adam kernels, so it is pinned first.
"""
import numpy as np

from oracle import mlp_oracle as M


def test_param_count():
    assert M.NPARAM == 128 * 64 + 128 + 2 * (128 * 128 + 128) + 4 * 128 + 4 == 41860


def test_backward_matches_central_differences():
    rng = np.random.default_rng(3)
    p = M.init(1) * 0.5
    p[M.NPARAM - 4:] = rng.normal(size=4) * 0.1                 # nonzero b4
    X = rng.normal(size=(7, M.IN))
    dout = rng.normal(size=(7, M.OUT))
    out, cache = M.forward(p, X)
    g = M.backward(p, cache, dout)
    idx = rng.choice(M.NPARAM, 60, replace=False)
    # include every parameter block
    starts = np.cumsum([0] + [int(np.prod(s)) for _, s in M.SHAPES])[:-1]
    idx = np.concatenate([idx, starts, starts + 1])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = ((M.forward(pp, X)[0] - M.forward(pm, X)[0]) * dout).sum() / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_gelu_grad_matches_central_differences():
    z = np.linspace(-6, 6, 101)
    fd = (M.gelu(z + 1e-6) - M.gelu(z - 1e-6)) / 2e-6
    assert np.abs(fd - M.gelu_grad(z)).max() < 1e-8


def test_mse_gradient():
    rng = np.random.default_rng(5)
    out, tgt = rng.normal(size=(9, 4)), rng.normal(size=(9, 4))
    loss, d = M.mse(out, tgt)
    assert np.all(d[:, 3] == 0)
    for (r, c) in [(0, 0), (4, 2), (8, 1)]:
        o2 = out.copy()
        o2[r, c] += 1e-6
        o3 = out.copy()
        o3[r, c] -= 1e-6
        fd = (M.mse(o2, tgt)[0] - M.mse(o3, tgt)[0]) / 2e-6
        assert abs(fd - d[r, c]) < 1e-8


def test_adam_first_step_is_signed_lr():
    # with bias correction the first step is -lr * g / (|g| + eps') ~ -lr * sign(g)
    g = np.array([1e-3, -2.0, 5.0])
    p, m, v = M.adam(np.zeros(3), g, np.zeros(3), np.zeros(3), 0.01, 0.9, 0.999, 1e-12, 1)
    assert np.allclose(p, -0.01 * np.sign(g), rtol=1e-6)
