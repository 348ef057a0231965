"""The allocation-free energy entry point (fipc_compute_energy_noalloc).

It serves callers that cannot allocate device memory while running (an application that owns
all device memory in one arena and forbids cudaMalloc after start-up).  The GPU cases call it
through the C ABI and compare with the context-based fipc_compute_energy on the same state, on
two calls in a row: both within 1e-10 relative, the two calls bitwise equal.  One state is
small (two cubes with six of the seven lists populated); one has tens of thousands of tets, so
the partial sums of many blocks are summed.  With all sizes zero the result is exactly 0.  The
argument checks (capacity, alignment) run on the host before anything is launched; the
alignment case needs no GPU.  This file sorts last so that a run stopping at the first failure
has already run every other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

D = ctypes.c_double


def P(t):
    return ctypes.c_void_p(t.data_ptr())


def _noalloc_vs_context(sim, scene):
    """Energy of sim's current state through the no-alloc entry point (two calls) and through
    the context; returns (e_noalloc[2], e_context)."""
    import torch
    from fastipc_gb300 import _native
    counts = sim.find_constraints()
    e_ctx = sim.compute_energy()
    dev = sim.device
    rest = scene.x
    tets = scene.tets.astype(np.int32)
    Dm = np.stack([rest[tets[:, 1]] - rest[tets[:, 0]], rest[tets[:, 2]] - rest[tets[:, 0]],
                   rest[tets[:, 3]] - rest[tets[:, 0]]], axis=2)
    nT = len(tets)
    lam = np.full(nT, scene.E * scene.nu / ((1 + scene.nu) * (1 - 2 * scene.nu)))
    mu = np.full(nT, scene.E / (2 * (1 + scene.nu)))

    def cu(a, dtype=torch.float64):
        return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype).contiguous()

    mass = cu(sim.mass())
    t_tets = cu(tets, torch.int32)
    dminv = cu(np.linalg.inv(Dm).reshape(nT, 9))
    vol = cu(np.linalg.det(Dm) / 3.0 / 2.0)
    t_lam, t_mu = cu(lam), cu(mu)
    x0 = cu(rest)
    rows = []
    for r in sim.constraints():
        r4 = np.zeros((max(len(r), 1), 4), np.int32)
        r4[:len(r), :r.shape[1]] = r
        rows.append(cu(r4, torch.int32))
    counts_h = (ctypes.c_int * 7)(*counts)
    rows_h = (ctypes.c_void_p * 7)(*[r.data_ptr() for r in rows])
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    L = _native.lib()
    for k in range(2):
        st = L.fipc_compute_energy_noalloc(sim.nV, P(sim.x), P(sim.xTilde), P(mass), nT, P(t_tets), P(dminv), P(vol), P(t_lam),
                                           P(t_mu), D(sim.dt), counts_h, rows_h, P(x0), D(sim.dhat2), D(sim.kappa),
                                           ctypes.c_void_p(out.data_ptr() + 8 * k), _native.stream())
        assert st == 0, _native.STATUS.get(st, st)
    torch.cuda.synchronize()
    return out.cpu().numpy(), e_ctx, counts


@pytest.mark.gpu
def test_noalloc_energy_matches_context_energy(newton_golden):
    import torch
    from fastipc_gb300 import scenes
    from fastipc_gb300.newton import NewtonIPC
    g = newton_golden
    scene = scenes.predeform(scenes.two_cubes(n=int(g['n']), seed=int(g['seed'])), float(g['predeform']), int(g['seed']))
    sim = NewtonIPC(scene)
    # a state with rows in six of the seven lists (the third recorded Newton iterate)
    sim.x.copy_(torch.from_numpy(g['it2_x']))
    sim.xTilde.copy_(torch.from_numpy(g['it2_xtilde']))
    e, e_ctx, counts = _noalloc_vs_context(sim, scene)
    assert sum(counts) > 0
    assert abs(e[0] - e_ctx) <= 1e-10 * abs(e_ctx), (e[0], e_ctx)
    assert abs(e[1] - e_ctx) <= 1e-10 * abs(e_ctx), (e[1], e_ctx)
    assert e[0] == e[1]
    sim.close()


@pytest.mark.gpu
def test_noalloc_energy_many_blocks():
    """A 48k-tet twisted bar a few steps into its twist: hundreds of partial sums."""
    from fastipc_gb300 import scenes
    from fastipc_gb300.newton import NewtonIPC
    scene = scenes.twisted_bar(nx=20, ny=20, nz=20, size=(0.05, 0.05, 0.05), seed=2)
    sim = NewtonIPC(scene, pcg_rtol=1e-8)
    for f in range(3):
        sim.step(f)
    sim.compute_xn_and_xTilde()
    assert scene.n_tets >= 40000
    e, e_ctx, _ = _noalloc_vs_context(sim, scene)
    assert abs(e[0] - e_ctx) <= 1e-10 * abs(e_ctx), (e[0], e_ctx)
    assert e[0] == e[1]
    sim.close()


@pytest.mark.gpu
def test_noalloc_energy_of_nothing_is_zero():
    import torch
    from fastipc_gb300 import _native
    out = torch.full((1,), 7.0, dtype=torch.float64, device='cuda:0')
    counts_h = (ctypes.c_int * 7)(0, 0, 0, 0, 0, 0, 0)
    for _ in range(2):
        st = _native.lib().fipc_compute_energy_noalloc(0, None, None, None, 0, None, None, None, None, None, D(0.01),
                                                       counts_h, None, None, D(1e-6), D(1.0), P(out), _native.stream())
        assert st == 0
        torch.cuda.synchronize()
        assert float(out.item()) == 0.0


@pytest.mark.gpu
def test_noalloc_rejects_requests_beyond_its_scratch():
    import torch
    from fastipc_gb300 import _native
    counts_h = (ctypes.c_int * 7)(0, 0, 0, 0, 0, 0, 0)
    dummy = torch.zeros(1, dtype=torch.float64, device='cuda:0')
    # 2^31 - 1 tets need far more than 65,536 partial sums: status 1 before anything runs
    st = _native.lib().fipc_compute_energy_noalloc(0, None, None, None, 2 ** 31 - 1, None, None, None, None, None, D(0.01),
                                                   counts_h, None, None, D(1e-6), D(1.0), P(dummy), _native.stream())
    assert st == 1


def test_noalloc_rejects_misaligned_pointers():
    """Misaligned tets, rows or doubles return status 5 before any CUDA call: the pointers below
    are never dereferenced, so this runs without a GPU."""
    from fastipc_gb300 import _native
    L = _native.lib()
    V = ctypes.c_void_p
    base = 1 << 20                              # a 256-aligned address value, never read
    ok = dict(x=V(base), xt=V(base + 256), m=V(base + 512), tets=V(base + 768), dminv=V(base + 1024), vol=V(base + 1280),
              lam=V(base + 1536), mu=V(base + 1792), x0=V(base + 2048), out=V(base + 2304))

    def call(counts, rows, **kw):
        a = dict(ok, **kw)
        counts_h = (ctypes.c_int * 7)(*counts)
        rows_h = (V * 7)(*rows) if rows is not None else None
        return L.fipc_compute_energy_noalloc(4, a['x'], a['xt'], a['m'], 1, a['tets'], a['dminv'], a['vol'], a['lam'], a['mu'],
                                             D(0.01), counts_h, rows_h, a['x0'], D(1e-6), D(1.0), a['out'], V(0))

    assert call([0] * 7, None, tets=V(base + 8)) == 5          # int4 tet loads: 16-byte
    assert call([0] * 7, None, x=V(base + 4)) == 5             # doubles: 8-byte
    assert call([0] * 7, None, out=V(base + 2)) == 5
    assert call([0, 0, 3, 0, 0, 0, 0], [base, base, base + 24, base, base, base, base]) == 5   # PT rows at 8 mod 16
