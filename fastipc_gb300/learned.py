"""Learned Newton warm start: a per-vertex MLP corrects the inertial guess of each time step.

The network (55 inputs -> 128 -> 128 -> 128 -> 3, GELU, FP32) runs and trains on the
hand-written CUDA kernels of libfastipc.so: features, forward, backward, MSE and Adam.  Torch
only holds the buffers.

Guess used by ``NewtonIPC.step`` after ``move_nodes`` (the reference starts Newton at x^n):
1. The inertial predictor d0 = xTilde - x^n on free vertices (x^n + dt v + dt^2 g).
2. The learned displacement d = d0 + s h out, with out the network's output, h the hash cell
   (mean boundary edge length) and s the target scale fixed at training time.
3. Each candidate step is filtered like a Newton direction.  alpha comes from the CCD and
   inversion filter, and is halved while any edge crosses a triangle.
4. Start from whichever of x^n, the filtered inertial step and the filtered learned step has the
   lowest incremental potential.  The learned guess falls back to the inertial one, and that
   one to the reference's x^n.
5. Newton then runs to the reference's unchanged tolerance.  A guess never admits intersection
   and never raises the starting energy.

Training data are transitions (x^n, v^n) -> x^{n+1} generated by the plain solver.  The
target per free vertex is (x^{n+1} - xTilde) / (s h): the part of the step that inertia does
not predict.  The last layer starts at zero, so an untrained network gives the inertial guess.
"""
import ctypes
import json
import time

import numpy as np
import torch

from . import _native as N
from ._native import check

F32 = torch.float32


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _log(msg):
    print(msg, flush=True)


class WarmStartMLP:
    IN, H, OUT = 64, 128, 4

    def __init__(self, device='cuda:0', seed=0, params=None, scale=1.0, rest_relative=True):
        self.scale = float(scale)
        self.rest_relative = bool(rest_relative)   # the feature mode it was trained with
        self.device = torch.device(device)
        self.nparam = int(N.lib().fipc_mlp_param_count())
        if params is None:
            from_np = _init_params(seed)
            params = torch.tensor(from_np, dtype=F32)
        self.params = params.to(self.device, F32).contiguous()
        assert self.params.numel() == self.nparam
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.t = 0
        self._scratch_n = 0

    def _scratch(self, n):
        if n > self._scratch_n:
            dev = self.device
            self.Z = torch.empty(3 * n * self.H, dtype=F32, device=dev)
            self.A = torch.empty(3 * n * self.H, dtype=F32, device=dev)
            self.dA = torch.empty(2 * n * self.H, dtype=F32, device=dev)
            self.out = torch.empty((n, self.OUT), dtype=F32, device=dev)
            self.dout = torch.empty((n, self.OUT), dtype=F32, device=dev)
            self.part = torch.empty((n + 255) // 256 + 1, dtype=F32, device=dev)
            self.loss = torch.empty(1, dtype=F32, device=dev)
            self._scratch_n = n

    def forward(self, X):
        n = X.shape[0]
        self._scratch(n)
        check(N.lib().fipc_mlp_forward(n, _p(X), _p(self.params), _p(self.Z), _p(self.A), _p(self.out), N.stream()), 'mlp_forward')
        return self.out[:n]

    def train_step(self, X, Y, lr=1e-3):
        """One Adam step on the mean squared error of batch (X [n,64], Y [n,4]); returns the loss."""
        n = X.shape[0]
        self.forward(X)
        L = N.lib()
        check(L.fipc_mlp_mse(n, _p(self.out), _p(Y), _p(self.dout), _p(self.part), _p(self.loss), N.stream()), 'mlp_mse')
        check(L.fipc_mlp_backward(n, _p(X), _p(self.params), _p(self.Z), _p(self.A), _p(self.dout), _p(self.grads), _p(self.dA),
                                  N.stream()), 'mlp_backward')
        self.t += 1
        check(L.fipc_mlp_adam(self.nparam, _p(self.params), _p(self.grads), _p(self.m), _p(self.v), ctypes.c_float(lr),
                              ctypes.c_float(0.9), ctypes.c_float(0.999), ctypes.c_float(1e-8), self.t, N.stream()), 'mlp_adam')
        return self.loss

    def save(self, path):
        np.savez(path, params=self.params.cpu().numpy(), scale=np.float64(self.scale), rest_relative=np.int32(self.rest_relative))

    @classmethod
    def load(cls, path, device='cuda:0'):
        d = np.load(path)
        return cls(device=device, params=torch.from_numpy(d['params']), scale=float(d['scale']),
                   rest_relative=bool(d['rest_relative']) if 'rest_relative' in d else False)


def _init_params(seed):
    rng = np.random.default_rng(seed)
    parts = []
    for name, shp in [('W1', (128, 64)), ('b1', (128,)), ('W2', (128, 128)), ('b2', (128,)), ('W3', (128, 128)), ('b3', (128,)),
                      ('W4', (4, 128)), ('b4', (4,))]:
        if name.startswith('W'):
            w = rng.normal(size=shp) * np.sqrt(2.0 / shp[1])
            parts.append(w * 0.0 if name == 'W4' else w)
        else:
            parts.append(np.zeros(shp))
    return np.concatenate([a.ravel() for a in parts]).astype(np.float32)


def features(sim, X=None, rest_relative=True):
    """Per-vertex inputs at the current state (constraint lists of the last find_constraints);
    one-ring positions relative to the rest shape's (the local deformation) by default."""
    if X is None:
        X = torch.empty((sim.nV, WarmStartMLP.IN), dtype=F32, device=sim.device)
    h = 1.0 / sim.inv_dx
    check(N.lib().fipc_mlp_features(sim.ctx, N.dptr(sim.x, torch.float64), N.dptr(sim.v, torch.float64),
                                    N.dptr(sim.dx_prev, torch.float64), ctypes.c_double(h), int(rest_relative), _p(X),
                                    N.stream()), 'mlp_features')
    return X


class LearnedStart:
    """``NewtonIPC.initial_guess`` hook: the lowest-energy filtered start among x^n, the inertial
    step and (kind 'mlp') the learned step.

    ``chosen`` counts which candidate each step started from; ``alphas`` the filtered step
    lengths of the chosen candidates.
    """

    def __init__(self, model=None, kind='mlp', smooth=4):
        assert kind in ('mlp', 'inertial')
        assert kind == 'inertial' or model is not None
        self.model, self.kind, self.smooth = model, kind, smooth
        self._tmp = None
        self.chosen = {'plain': 0, 'inertial': 0, 'mlp': 0}
        self.alphas = []
        self._X = None

    @property
    def accepted(self):
        return self.chosen['inertial'] + self.chosen['mlp']

    @property
    def fallback(self):
        return self.chosen['plain']

    def inertial(self, sim):
        free = (sim.fixed == 0).unsqueeze(1)
        return torch.where(free, sim.xTilde - sim.x, torch.zeros_like(sim.x))

    def learned(self, sim, d0):
        """d0 + S(s h out), S = ``smooth`` passes of one-ring averaging; needs the constraint
        lists of the current positions (features)."""
        if self._X is None or self._X.shape[0] != sim.nV:
            self._X = torch.empty((sim.nV, WarmStartMLP.IN), dtype=F32, device=sim.device)
            self._tmp = torch.empty((sim.nV, 3), dtype=torch.float64, device=sim.device)
        X = features(sim, self._X, self.model.rest_relative)
        out = self.model.forward(X)
        corr = torch.where((sim.fixed == 0).unsqueeze(1), out[:, :3].to(torch.float64) * (self.model.scale / sim.inv_dx),
                           torch.zeros_like(d0)).contiguous()
        if self.smooth:
            check(N.lib().fipc_mlp_smooth(sim.ctx, N.dptr(sim.fixed, torch.uint8), N.dptr(corr, torch.float64),
                                          N.dptr(self._tmp, torch.float64), int(self.smooth), N.stream()), 'mlp_smooth')
        return d0 + corr

    def _filtered(self, sim, d):
        """x = x^n + alpha d with alpha from the CCD filter and collision halving; its energy."""
        sim.data_sol.copy_(d)
        alpha = sim.compute_intersection_free_step_size()
        sim.apply_sol(alpha)
        k = 0
        while sim.check_collision():
            alpha /= 2.0
            sim.apply_sol(alpha)
            k += 1
            if k > sim.max_halvings:
                return None, None
        sim.find_constraints()
        return alpha, sim.compute_energy()

    def __call__(self, sim, f):
        sim.find_constraints()
        e_best, name_best, d_best, a_best = sim.compute_energy(), 'plain', None, 0.0
        sim.save_xPrev()
        d0 = self.inertial(sim)
        cands = [('inertial', d0)]
        if self.kind == 'mlp':
            cands.append(('mlp', self.learned(sim, d0)))   # features at x^n (lists found above)
        for name, d in cands:
            alpha, e = self._filtered(sim, d)
            if alpha is not None and e < e_best:
                e_best, name_best, d_best, a_best = e, name, d, alpha
        if d_best is None:
            sim.x.copy_(sim.xPrev)
        else:
            sim.data_sol.copy_(d_best)
            sim.apply_sol(a_best)
            self.alphas.append(a_best)
        self.chosen[name_best] += 1


# ---------------------------------------------------------------------- data and training
class BatchLearnedStart:
    """``BatchNewtonIPC.initial_guess`` hook: for every scene of a batch, the lowest-energy
    filtered start among x^n, the inertial step and (kind 'mlp') the learned step, exactly as
    ``LearnedStart`` chooses for one scene.  Every scene gets its own CCD step, collision halving
    and choice.  The network's inputs are divided by one cell size, so the scenes of the batch
    must share it (same mesh resolution)."""

    def __init__(self, model=None, kind='mlp', smooth=4, max_halvings=64):
        assert kind in ('mlp', 'inertial')
        assert kind == 'inertial' or model is not None
        self.model, self.kind, self.smooth, self.max_halvings = model, kind, smooth, max_halvings
        self.chosen = {'plain': 0, 'inertial': 0, 'mlp': 0}
        self._X = self._tmp = None

    def _learned(self, sim, d0, free):
        if not np.allclose(sim.inv_dx, sim.inv_dx[0], rtol=1e-12):
            raise ValueError('the learned start needs scenes with one cell size')
        if self._X is None or self._X.shape[0] != sim.nV:
            self._X = torch.empty((sim.nV, WarmStartMLP.IN), dtype=F32, device=sim.device)
            self._tmp = torch.empty((sim.nV, 3), dtype=torch.float64, device=sim.device)
        h = 1.0 / float(sim.inv_dx[0])
        check(N.lib().fipc_mlp_features(sim.ctx, N.dptr(sim.x, torch.float64), N.dptr(sim.v, torch.float64),
                                        N.dptr(sim.dx_prev, torch.float64), ctypes.c_double(h), int(self.model.rest_relative),
                                        _p(self._X), N.stream()), 'mlp_features')
        out = self.model.forward(self._X)
        corr = torch.where(free, out[:, :3].to(torch.float64) * (self.model.scale * h), torch.zeros_like(d0)).contiguous()
        if self.smooth:
            check(N.lib().fipc_mlp_smooth(sim.ctx, N.dptr(sim.fixed, torch.uint8), N.dptr(corr, torch.float64),
                                          N.dptr(self._tmp, torch.float64), int(self.smooth), N.stream()), 'mlp_smooth')
        return d0 + corr

    def __call__(self, sim, f):
        sim.find_constraints()
        e_best = sim.compute_energy(torch.empty_like(sim.E)).clone()
        choice = torch.zeros(sim.S, dtype=torch.int64, device=sim.device)
        a_best = torch.zeros_like(sim.alpha)
        sim.save_xPrev()
        free = (sim.fixed == 0).unsqueeze(1)
        d0 = torch.where(free, sim.xTilde - sim.x, torch.zeros_like(sim.x))
        cands = [d0]
        if self.kind == 'mlp':
            cands.append(self._learned(sim, d0, free))   # features at x^n (lists found above)
        for idx, d in enumerate(cands, start=1):
            sim.data_sol.copy_(d)
            sim.compute_intersection_free_step_size()
            sim.apply_sol()
            valid = np.ones(sim.S, bool)
            for _ in range(self.max_halvings + 1):
                hit = sim.check_collision()
                if not hit.any():
                    break
                sim._halve(hit)
            valid &= ~sim.check_collision()
            sim.find_constraints()
            e = sim.compute_energy()
            better = torch.from_numpy(valid).to(sim.device) & (e < e_best)
            e_best = torch.where(better, e, e_best)
            choice = torch.where(better, torch.full_like(choice, idx), choice)
            a_best = torch.where(better, sim.alpha, a_best)
        cv = choice[sim.v_scene].unsqueeze(1)
        d = torch.zeros_like(sim.x)
        for idx, c in enumerate(cands, start=1):
            d = torch.where(cv == idx, c, d)
        sim.data_sol.copy_(d)
        sim.alpha.copy_(a_best)
        sim.apply_sol()
        counts = torch.bincount(choice, minlength=3).cpu().numpy()
        for k, name in enumerate(('plain', 'inertial', 'mlp')):
            self.chosen[name] += int(counts[k])


class _Recorder:
    """Hook that records (features, free mask, inertial predictor) at each step's start."""

    def __init__(self, inner=None, rest_relative=True):
        self.pending = None
        self.inner = inner
        self.rest_relative = rest_relative

    def __call__(self, sim, f):
        sim.find_constraints()
        self.pending = (features(sim, rest_relative=self.rest_relative).clone(), (sim.fixed == 0).clone(), sim.xTilde.clone())
        if self.inner is not None:
            self.inner(sim, f)


def collect(scene, steps, device='cuda:0', pcg_rtol=1e-6, start=0, rest_relative=True, stride=1):
    """Run the solver (inertial start, which converges to the same steps as the plain one) for
    ``steps`` steps; returns (X [n,64], Y [n,4]) over the free vertices of every stride-th step
    from start on, Y = (x^{n+1} - xTilde) / h."""
    from .newton import NewtonIPC
    sim = NewtonIPC(scene, device=device, pcg_rtol=pcg_rtol)
    rec = _Recorder(LearnedStart(kind='inertial'), rest_relative=rest_relative)
    sim.initial_guess = rec
    h = 1.0 / sim.inv_dx
    Xs, Ys = [], []
    for f in range(steps):
        sim.step(f)
        if f < start or (f - start) % stride:
            continue
        X, free, xt = rec.pending
        Y = torch.zeros((sim.nV, 4), dtype=F32, device=sim.device)
        Y[:, :3] = ((sim.x - xt) / h).to(F32)
        Xs.append(X[free])
        Ys.append(Y[free])
    sim.close()
    return torch.cat(Xs), torch.cat(Ys)


def train(model, X, Y, epochs=30, batch=8192, lr=1e-3, seed=0, log=None):
    """Mini-batch Adam on the CUDA kernels with a cosine learning-rate decay."""
    g = torch.Generator(device='cpu').manual_seed(seed)
    n = X.shape[0]
    nb = max(1, n // batch)
    total = epochs * nb
    step = 0
    hist = []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g).to(X.device)
        acc = torch.zeros((), device=X.device)
        for b in range(nb):
            idx = perm[b * batch:(b + 1) * batch]
            cur = lr * 0.5 * (1 + np.cos(np.pi * step / total))
            acc += model.train_step(X[idx].contiguous(), Y[idx].contiguous(), lr=cur)[0]
            step += 1
        hist.append(float(acc) / nb)
        if log:
            log(f'epoch {ep} loss {hist[-1]:.4e}')
    return hist


def evaluate(model, X, Y):
    out = model.forward(X)
    return float(((out[:, :3] - Y[:, :3]) ** 2).mean())


def _result(sim, guess, steps, wall, intersect):
    out = {'steps': steps, 'newton': int(sum(sim.newton_iters)), 'pcg': int(sum(sim.pcg_iters)), 'wall_s': wall,
           'intersecting_steps': intersect, 'newton_per_step': list(map(int, sim.newton_iters))}
    if guess is not None:
        out['chosen'] = dict(guess.chosen)
    return out


def run_scene(scene, steps, guess=None, device='cuda:0', pcg_rtol=1e-6):
    """Plain (guess None) or guessed run; returns counters and the final positions."""
    from .newton import NewtonIPC
    sim = NewtonIPC(scene, device=device, pcg_rtol=pcg_rtol)
    sim.initial_guess = guess
    intersect = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for f in range(steps):
        sim.step(f)
        intersect += int(sim.check_collision())
    torch.cuda.synchronize()
    out = _result(sim, guess, steps, time.perf_counter() - t0, intersect)
    x = sim.x.cpu().numpy()
    sim.close()
    return out, x


def _split(X, Y, seed=0):
    g = torch.Generator(device='cpu').manual_seed(seed)
    perm = torch.randperm(X.shape[0], generator=g).to(X.device)
    nval = X.shape[0] // 10
    return X[perm[nval:]].contiguous(), Y[perm[nval:]].contiguous(), X[perm[:nval]].contiguous(), Y[perm[:nval]].contiguous()


def fit(X, Y, device='cuda:0', epochs=30, log=_log, seed=0, rest_relative=True):
    """Train a model on (X, Y in h units); the target scale is the RMS of Y.  Returns the model
    and its statistics (validation MSE of the network and of the inertial guess, in h^2)."""
    Xt, Yt, Xv, Yv = _split(X, Y, seed)
    scale = float(Yt[:, :3].pow(2).mean().sqrt())
    model = WarmStartMLP(device, seed=seed, scale=scale, rest_relative=rest_relative)
    t1 = time.perf_counter()
    hist = train(model, Xt, Yt / scale, epochs=epochs, log=log)
    torch.cuda.synchronize()
    stats = {'rows_train': int(Xt.shape[0]), 'rows_val': int(Xv.shape[0]), 'train_s': time.perf_counter() - t1, 'scale_h': scale,
             'loss_hist': hist, 'val_mse_h2': evaluate(model, Xv, Yv / scale) * scale ** 2,
             'val_mse_h2_inertial': float(Yv[:, :3].pow(2).mean())}
    return model, stats


def collect_bar(nx, seed, steps, device='cuda:0', rest_relative=True, pcg_rtol=1e-6, stride=1):
    """Transitions of the twisted bar (20 x 20 cross-section, nx hexes long) with the inertial start."""
    from . import scenes as S
    sc = S.twisted_bar(nx=nx, ny=20, nz=20, size=(nx / 400.0, 0.05, 0.05), seed=seed)
    return collect(sc, steps, device, pcg_rtol, rest_relative=rest_relative, stride=stride)


def compare_starts(sim, steps, f0, modes, log=_log, warmup=1):
    """Run steps [f0, f0 + steps) from sim's current state once per mode (the state is restored
    between modes).  modes: name -> None (plain) or a LearnedStart.  Before the timed runs every
    mode takes `warmup` untimed steps from the same state, so that first-use costs (buffer
    growth for a large-motion CCD grid, the network's first launches) fall outside every mode's
    wall time."""
    snap = (sim.x.clone(), sim.v.clone(), sim.dx_prev.clone())
    out, xs = {}, {}
    for name, guess in modes.items():
        sim.initial_guess = guess
        for k in range(warmup):
            if k == 0:
                sim.x.copy_(snap[0])
                sim.v.copy_(snap[1])
                sim.dx_prev.copy_(snap[2])
            sim.step(f0 + k)
    for name, guess in modes.items():
        sim.x.copy_(snap[0])
        sim.v.copy_(snap[1])
        sim.dx_prev.copy_(snap[2])
        sim.newton_iters, sim.pcg_iters = [], []
        sim.initial_guess = guess
        inter = 0
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for f in range(f0, f0 + steps):
            sim.step(f)
            inter += int(sim.check_collision())
        torch.cuda.synchronize()
        out[name] = _result(sim, guess, steps, time.perf_counter() - t1, inter)
        xs[name] = sim.x.cpu().numpy()
        if log:
            log(f"{name}: newton {out[name]['newton']} pcg {out[name]['pcg']} wall {out[name]['wall_s']:.2f} s")
    first = next(iter(xs))
    for name in out:
        out[name]['max_dev_vs_' + first] = float(np.abs(xs[name] - xs[first]).max())
    sim.initial_guess = None
    return out


def experiment_bar(out_dir, nx=400, train_seed=1, train_steps=80, eval_seed=0, eval_start=20, eval_steps=40, device='cuda:0',
                   epochs=15, rest_relative=True, log=_log, pcg_rtol=1e-6, stride=1, smooth=(0, 2, 4, 8)):
    """Train on the transitions of one twisted bar (jitter seed train_seed) and compare plain /
    inertial / learned starts on another (eval_seed), over steps [eval_start, eval_start +
    eval_steps) from one state."""
    import os
    from . import scenes as S
    from .newton import NewtonIPC
    os.makedirs(out_dir, exist_ok=True)
    t0 = time.perf_counter()
    X, Y = collect_bar(nx, train_seed, train_steps, device, rest_relative, pcg_rtol, stride)
    res = {'nx': nx, 'train_seed': train_seed, 'train_steps': train_steps, 'stride': stride, 'eval_seed': eval_seed, 'eval_start': eval_start,
           'eval_steps': eval_steps, 'rest_relative': rest_relative, 'collect_s': time.perf_counter() - t0}
    model, stats = fit(X, Y, device, epochs, log, rest_relative=rest_relative)
    del X, Y
    res.update(stats)
    tag = 'rr' if rest_relative else 'cur'
    model.save(os.path.join(out_dir, f'warmstart_bar{nx}_{tag}.npz'))
    sc = S.twisted_bar(nx=nx, ny=20, nz=20, size=(nx / 400.0, 0.05, 0.05), seed=eval_seed)
    sim = NewtonIPC(sc, device=device, pcg_rtol=pcg_rtol)
    sim.initial_guess = LearnedStart(kind='inertial')
    for f in range(eval_start):
        sim.step(f)
    modes = {'plain': None, 'inertial': LearnedStart(kind='inertial')}
    for k in smooth:
        modes[f'mlp_s{k}'] = LearnedStart(model, kind='mlp', smooth=k)
    res['eval'] = compare_starts(sim, eval_steps, eval_start, modes, log)
    sim.close()
    with open(os.path.join(out_dir, f'warmstart_bar{nx}_{tag}.json'), 'w') as fh:
        json.dump(res, fh, indent=1)
    return res


def experiment_drops(out_dir, n_train=40, n_eval=10, steps=30, m=2, n=4, device='cuda:0', epochs=15, rest_relative=True,
                     smooth=4, log=_log, pcg_rtol=1e-6):
    """Lattice drops in the style of the 216-cube configuration (m^3 cubes of n^3 hexes over a
    ground box): train on seeds [0, n_train), compare starts on seeds [1000, 1000 + n_eval)."""
    import os
    from . import scenes as S
    from .newton import NewtonIPC
    os.makedirs(out_dir, exist_ok=True)
    t0 = time.perf_counter()
    Xs, Ys = [], []
    for seed in range(n_train):
        X, Y = collect(S.cube_lattice(m=m, n=n, seed=seed), steps, device, pcg_rtol, rest_relative=rest_relative)
        Xs.append(X)
        Ys.append(Y)
    res = {'m': m, 'n': n, 'n_train': n_train, 'n_eval': n_eval, 'steps': steps, 'rest_relative': rest_relative,
           'transitions': n_train * steps, 'collect_s': time.perf_counter() - t0}
    model, stats = fit(torch.cat(Xs), torch.cat(Ys), device, epochs, log, rest_relative=rest_relative)
    del Xs, Ys
    res.update(stats)
    model.save(os.path.join(out_dir, f'warmstart_drops_m{m}n{n}.npz'))
    tot = {}
    for seed in range(1000, 1000 + n_eval):
        sim = NewtonIPC(S.cube_lattice(m=m, n=n, seed=seed), device=device, pcg_rtol=pcg_rtol)
        r = compare_starts(sim, steps, 0, {'plain': None, 'inertial': LearnedStart(kind='inertial'),
                                           'mlp': LearnedStart(model, kind='mlp', smooth=smooth)}, log=None)
        sim.close()
        for k, v in r.items():
            t = tot.setdefault(k, {'newton': 0, 'pcg': 0, 'wall_s': 0.0, 'intersecting_steps': 0})
            for q in t:
                t[q] += v[q]
        log(f"seed {seed}: " + ', '.join(f"{k} {v['newton']}" for k, v in r.items()))
    res['eval'] = tot
    with open(os.path.join(out_dir, f'warmstart_drops_m{m}n{n}.json'), 'w') as fh:
        json.dump(res, fh, indent=1)
    return res


def evaluate_drops_batched(model, n_eval=20, steps=30, m=2, n=4, first_seed=1000, smooth=4, device='cuda:0', pcg_rtol=1e-6,
                           log=_log):
    """Plain / inertial / learned starts on n_eval unseen lattice drops stepped together in one
    batch context (each scene keeps its own Newton loop and its own start choice)."""
    from . import scenes as S
    from .batch import BatchNewtonIPC
    scs = [S.cube_lattice(m=m, n=n, seed=first_seed + k) for k in range(n_eval)]
    sim = BatchNewtonIPC(scs, device=device, pcg_rtol=pcg_rtol)
    x0, v0 = sim.x.clone(), sim.v.clone()
    res = {}
    for name, guess in (('plain', None), ('inertial', BatchLearnedStart(kind='inertial')),
                        ('learned', BatchLearnedStart(model, kind='mlp', smooth=smooth))):
        sim.x.copy_(x0)
        sim.v.copy_(v0)
        sim.dx_prev.zero_()
        sim.newton_iters = []
        sim.initial_guess = guess
        inter = 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for f in range(steps):
            sim.step(f)
            inter += int(sim.check_collision().sum())
        torch.cuda.synchronize()
        its = np.stack(sim.newton_iters)
        res[name] = {'newton': int(its.sum()), 'newton_per_scene_step': float(its.mean()), 'wall_s': time.perf_counter() - t0,
                     'intersecting_scene_steps': inter, 'chosen': dict(guess.chosen) if guess else None}
        if log:
            log(f"{name}: newton {res[name]['newton']} ({res[name]['newton_per_scene_step']:.2f} per scene-step) "
                f"wall {res[name]['wall_s']:.1f} s")
    sim.close()
    res['config'] = {'n_eval': n_eval, 'steps': steps, 'm': m, 'n': n, 'seeds': [first_seed, first_seed + n_eval - 1], 'smooth': smooth}
    return res


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description='train and evaluate the learned Newton warm start')
    ap.add_argument('--out', default='warmstart_out')
    ap.add_argument('--epochs', type=int, default=15)
    ap.add_argument('--bar', type=int, default=0, help='twisted bar with nx hexes along its axis (0: skip)')
    ap.add_argument('--train-seed', type=int, default=1)
    ap.add_argument('--train-steps', type=int, default=80)
    ap.add_argument('--stride', type=int, default=1, help='keep every stride-th training step')
    ap.add_argument('--smooth', default='0,2,4,8', help='smoothing passes to evaluate')
    ap.add_argument('--eval-start', type=int, default=20)
    ap.add_argument('--eval-steps', type=int, default=40)
    ap.add_argument('--current-relative', action='store_true', help='one-ring offsets x_j - x_i instead of rest-relative')
    ap.add_argument('--drops', type=int, default=0, help='lattice drops: number of training seeds (0: skip)')
    ap.add_argument('--drop-eval', type=int, default=10)
    ap.add_argument('--drop-steps', type=int, default=30)
    ap.add_argument('--drop-weights', default='', help='evaluate these weights on unseen drops (batched) instead of training')
    a = ap.parse_args(argv)
    rr = not a.current_relative
    if a.bar:
        experiment_bar(a.out, nx=a.bar, train_seed=a.train_seed, train_steps=a.train_steps, eval_start=a.eval_start,
                       eval_steps=a.eval_steps, epochs=a.epochs, rest_relative=rr, stride=a.stride,
                       smooth=tuple(int(k) for k in a.smooth.split(',')))
    if a.drop_weights:
        import os
        r = evaluate_drops_batched(WarmStartMLP.load(a.drop_weights), n_eval=a.drop_eval, steps=a.drop_steps)
        os.makedirs(a.out, exist_ok=True)
        with open(os.path.join(a.out, 'drops_eval.json'), 'w') as fh:
            json.dump(r, fh, indent=1)
    if a.drops:
        experiment_drops(a.out, n_train=a.drops, n_eval=a.drop_eval, steps=a.drop_steps, epochs=a.epochs, rest_relative=rr)


if __name__ == '__main__':
    main()
