"""The learned warm start on the GB300: CUDA MLP kernels against the numpy MLP oracle, the
per-vertex features against numpy, and the guard of the Newton start (never intersecting,
never above the plain start's energy, same converged step within the Newton tolerance).

Bars: forward 2e-5 and gradients 1e-4 relative to the largest entry (FP32 kernels against an
FP64 restatement), Adam 1e-6, features 1e-6."""
import ctypes

import numpy as np
import pytest
import torch

from fastipc_gb300 import scenes
from fastipc_gb300 import _native as NN
from fastipc_gb300.learned import LearnedStart, WarmStartMLP, collect, features, train
from fastipc_gb300.newton import NewtonIPC
from oracle import mlp_oracle as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu
F32 = torch.float32


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def relmax(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


@pytest.fixture(scope='module')
def params():
    p = M.init(2).astype(np.float32)
    rng = np.random.default_rng(9)
    p[-4:] = rng.normal(size=4).astype(np.float32) * 0.1
    return p


@pytest.mark.parametrize('n', [1, 63, 1000])
def test_forward_backward_match_oracle(params, n):
    rng = np.random.default_rng(n)
    X = rng.normal(size=(n, M.IN)).astype(np.float32)
    dout = rng.normal(size=(n, M.OUT)).astype(np.float32)
    model = WarmStartMLP('cuda:0', params=torch.from_numpy(params))
    Xd = torch.from_numpy(X).cuda()
    out = model.forward(Xd).cpu().numpy()
    ref, cache = M.forward(params.astype(np.float64), X.astype(np.float64))
    assert relmax(out, ref) < 2e-5
    model.dout[:n].copy_(torch.from_numpy(dout))
    st = NN.lib().fipc_mlp_backward(n, _p(Xd), _p(model.params), _p(model.Z), _p(model.A), _p(model.dout), _p(model.grads),
                                    _p(model.dA), NN.stream())
    assert st == 0
    g = model.grads.cpu().numpy()
    gref = M.backward(params.astype(np.float64), cache, dout.astype(np.float64))
    o = 0
    for name, shp in M.SHAPES:
        k = int(np.prod(shp))
        assert relmax(g[o:o + k], gref[o:o + k]) < 1e-4, name
        o += k


def test_mse_matches_oracle():
    rng = np.random.default_rng(4)
    n = 777
    out = rng.normal(size=(n, 4)).astype(np.float32)
    tgt = rng.normal(size=(n, 4)).astype(np.float32)
    o, t = torch.from_numpy(out).cuda(), torch.from_numpy(tgt).cuda()
    d = torch.empty_like(o)
    part = torch.empty(8, dtype=F32, device='cuda')
    loss = torch.empty(1, dtype=F32, device='cuda')
    assert NN.lib().fipc_mlp_mse(n, _p(o), _p(t), _p(d), _p(part), _p(loss), NN.stream()) == 0
    lref, dref = M.mse(out.astype(np.float64), tgt.astype(np.float64))
    assert abs(float(loss) - lref) < 1e-5 * lref
    assert relmax(d.cpu().numpy(), dref) < 1e-6


def test_adam_matches_oracle():
    rng = np.random.default_rng(8)
    n = 5000
    p, g, m = (rng.normal(size=n).astype(np.float32) for _ in range(3))
    v = rng.uniform(0.1, 2.0, n).astype(np.float32)
    P, G, Mm, V = (torch.from_numpy(a.copy()).cuda() for a in (p, g, m, v))
    st = NN.lib().fipc_mlp_adam(n, _p(P), _p(G), _p(Mm), _p(V), ctypes.c_float(1e-2), ctypes.c_float(0.9),
                                ctypes.c_float(0.999), ctypes.c_float(1e-8), 3, NN.stream())
    assert st == 0
    pr, mr, vr = M.adam(p.astype(np.float64), g.astype(np.float64), m.astype(np.float64), v.astype(np.float64), 1e-2, 0.9, 0.999,
                        1e-8, 3)
    assert relmax(P.cpu().numpy(), pr) < 1e-6
    assert relmax(Mm.cpu().numpy(), mr) < 1e-6
    assert relmax(V.cpu().numpy(), vr) < 1e-6


def test_argument_errors():
    L = NN.lib()
    z = ctypes.c_void_p(0)
    assert L.fipc_mlp_forward(-1, z, z, z, z, z, NN.stream()) != 0
    assert L.fipc_mlp_adam(10, z, z, z, z, ctypes.c_float(1e-3), ctypes.c_float(0.9), ctypes.c_float(0.999),
                           ctypes.c_float(1e-8), 0, NN.stream()) != 0
    X = torch.zeros((1, 64), dtype=F32, device='cuda')
    m = WarmStartMLP('cuda:0')
    assert L.fipc_mlp_forward(0, _p(X), _p(m.params), _p(X), _p(X), _p(X), NN.stream()) == 0   # empty batch


@pytest.fixture(scope='module')
def contact_sim():
    s = NewtonIPC(scenes.two_cubes(n=3, seed=2), pcg_rtol=1e-10)
    for f in range(3):
        s.step(f)
    s.find_constraints()
    yield s
    s.close()


@pytest.mark.parametrize('rest_relative', [False, True])
def test_features_match_numpy(contact_sim, rest_relative):
    s = contact_sim
    assert sum(s.counts) > 0, 'scene should be in contact'
    X = features(s, rest_relative=rest_relative).cpu().numpy()
    X0 = np.asarray(s.scene.x, np.float64)
    A, _, _ = s.export_system()
    rp, ci = A.indptr, A.indices
    x, v, dxp = s.x.cpu().numpy(), s.v.cpu().numpy(), s.dx_prev.cpu().numpy()
    assert np.abs(dxp).max() > 0
    h = 1.0 / s.inv_dx
    ref = np.zeros((s.nV, 64), np.float32)
    for i in range(s.nV):
        nb = [j for j in ci[rp[i]:rp[i + 1]] if j != i][:16]
        for k, j in enumerate(nb):
            d = x[j] - x[i]
            if rest_relative:
                d = d - (X0[j] - X0[i])
            ref[i, 3 * k:3 * k + 3] = (d * (1.0 / h)).astype(np.float32)
    ref[:, 48:51] = (v * s.dt * (1.0 / h)).astype(np.float32)
    ref[:, 51:54] = (dxp * (1.0 / h)).astype(np.float32)
    dmin = np.full(s.nV, np.inf, np.float32)
    rows = s.constraints()
    for t, r in enumerate(rows):
        if len(r) == 0:
            continue
        pick = {0: ([0, 1], 0), 1: ([0, 1, 2], 1), 2: ([0, 1, 2, 3], 2), 3: ([0, 1, 2, 3], 3), 4: ([0, 1, 2, 3], 3),
                5: ([0, 2], 0), 6: ([0, 2, 3], 1)}[t]
        pts = np.zeros((len(r), 4, 3))
        pts[:, :len(pick[0])] = x[r[:, pick[0]]]
        d2, _, _ = O.distance(pick[1], pts)
        dist = np.sqrt(np.maximum(d2, 0)).astype(np.float32)
        for k in range(r.shape[1]):
            np.minimum.at(dmin, r[:, k], dist)
    ref[:, 54] = np.minimum(dmin * np.float32(1.0 / float(s.scene.dhat)), np.float32(1.0))
    assert (ref[:, 54] < 1).any()
    np.testing.assert_allclose(X, ref, rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize('kind', ['inertial', 'mlp'])
def test_guess_is_safe_and_converges_to_the_same_step(kind):
    sc = scenes.two_cubes(n=4, seed=3)
    plain = NewtonIPC(sc, pcg_rtol=1e-10)
    guessed = NewtonIPC(sc, pcg_rtol=1e-10)
    model = None
    if kind == 'mlp':
        # an untrained network with a random last layer: a poor guess the filter must keep safe
        model = WarmStartMLP('cuda:0', seed=1, scale=0.5)
        g = torch.Generator(device='cpu').manual_seed(5)
        model.params[-516:] = torch.randn(516, generator=g).to(model.params)
    hook = LearnedStart(model, kind=kind)
    guessed.initial_guess = hook
    for f in range(4):
        plain.step(f)
        guessed.step(f)
        assert not guessed.check_collision()
        dev = (guessed.x - plain.x).abs().max().item()
        # Newton stops once its direction is below 1e-2 dt = 1e-4 (max norm), so two starts
        # land within about twice that of each other
        assert dev < 3e-4, (f, dev)
        # carry the same state on, so each step is compared from one start
        guessed.x.copy_(plain.x)
        guessed.v.copy_(plain.v)
        guessed.dx_prev.copy_(plain.dx_prev)
    assert hook.accepted + hook.fallback == 4
    plain.close()
    guessed.close()


def test_training_lowers_the_loss():
    X, Y = collect(scenes.two_cubes(n=3, seed=0), 6)
    assert X.shape[1] == 64 and X.shape[0] == Y.shape[0] > 0
    model = WarmStartMLP('cuda:0', seed=0)
    hist = train(model, X, Y, epochs=15, batch=256, lr=3e-3)
    assert hist[-1] < 0.5 * hist[0]


def test_trained_network_beats_the_starts_without_it():
    """What the trained network gains: the committed weights (trained on the twisted bar with
    jitter seed 1) on an unseen bar (seed 2), steps 0-99, against the same solver started from
    x^n (the reference) and from the filtered inertial guess, at the same Newton tolerance."""
    import os
    from fastipc_gb300.learned import compare_starts
    weights = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'fastipc_gb300', 'weights',
                           'warmstart_bar400.npz')
    model = WarmStartMLP.load(weights)
    sim = NewtonIPC(scenes.twisted_bar(seed=2), pcg_rtol=1e-6)
    r = compare_starts(sim, 100, 0, {'plain': None, 'inertial': LearnedStart(kind='inertial'),
                                     'learned': LearnedStart(model, kind='mlp', smooth=4)}, log=None)
    sim.close()
    assert all(v['intersecting_steps'] == 0 for v in r.values())
    assert r['learned']['newton'] < r['inertial']['newton'] < r['plain']['newton'], {k: v['newton'] for k, v in r.items()}
    assert r['learned']['newton'] <= 0.75 * r['plain']['newton']
