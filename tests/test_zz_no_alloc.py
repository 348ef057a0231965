"""The allocation-free energy entry point (fipc_compute_energy_noalloc) on the GPU.

It serves callers that cannot allocate device memory while running (an application that owns
all device memory in one arena and forbids cudaMalloc after start-up).  Checked through the C
ABI against the context-based fipc_compute_energy on the same state, on two calls in a row:
both within 1e-10 relative, the two calls bitwise equal.  This file sorts last so that a run
stopping at the first failure has already run every other test; it also passes on its own in
a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

from fastipc_gb300 import scenes
from fastipc_gb300.newton import NewtonIPC

pytestmark = pytest.mark.gpu
D = ctypes.c_double


def P(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_energy_matches_context_energy(newton_golden):
    from fastipc_gb300 import _native
    g = newton_golden
    scene = scenes.predeform(scenes.two_cubes(n=int(g['n']), seed=int(g['seed'])), float(g['predeform']), int(g['seed']))
    sim = NewtonIPC(scene)
    # a state with rows in six of the seven lists (the third recorded Newton iterate)
    sim.x.copy_(torch.from_numpy(g['it2_x']))
    sim.xTilde.copy_(torch.from_numpy(g['it2_xtilde']))
    counts = sim.find_constraints()
    assert sum(counts) > 0
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
    e = out.cpu().numpy()
    assert abs(e[0] - e_ctx) <= 1e-10 * abs(e_ctx), (e[0], e_ctx)
    assert abs(e[1] - e_ctx) <= 1e-10 * abs(e_ctx), (e[1], e_ctx)
    assert e[0] == e[1]
    sim.close()


def test_noalloc_rejects_requests_beyond_its_scratch():
    from fastipc_gb300 import _native
    counts_h = (ctypes.c_int * 7)(0, 0, 0, 0, 0, 0, 0)
    dummy = torch.zeros(1, dtype=torch.float64, device='cuda:0')
    # 2^31 - 1 tets need far more than 65,536 partial sums: status 1 before anything runs
    st = _native.lib().fipc_compute_energy_noalloc(0, None, None, None, 2 ** 31 - 1, None, None, None, None, None, D(0.01),
                                                   counts_h, None, None, D(1e-6), D(1.0), P(dummy), _native.stream())
    assert st == 1
