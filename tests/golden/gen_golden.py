"""Generate the golden fixtures under tests/golden/ from the REFERENCE's own code.

Runs only where the reference checkout exists (default /root/reference; override with
FASTIPC_REFERENCE).  The GPU machine never runs this; the tests only read the .npz files it wrote.

Sources of truth:
  * the reference's Python kernels (common/math/distance.py, ipc.py, math_tools.py,
    common/physics/neo_hookean.py, graph_tools.py, projects/FastIPC/NEWTON_IPC.py), executed
    through ``taichi_standin`` (Taichi itself is not installable here);
  * the reference's native ``a.so`` (common/math/wrapper/wrapper.cpp + EVCTCD/CTCD.cpp) built
    from source into oracle/_ref/ by ``oracle/build_ref.sh`` and called through ctypes, exactly
    as the reference's ``ti.external_func_call`` glue does.

Stand-ins (documented, not the reference's own code): Taichi's ``ti.svd`` (numpy SVD,
rotation-variant), CHOLMOD's ``cholesky(A)(b)`` (scipy ``splu``, exact sparse LU).

Usage:  python tests/golden/gen_golden.py [unit|newton|newton2d|all]
"""
import ctypes
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get('FASTIPC_REFERENCE', '/root/reference')
ASO = os.path.join(REPO, 'oracle', '_ref', 'a.so')
sys.path.insert(0, HERE)
sys.path.insert(0, REPO)

import taichi_standin as ti  # noqa: E402


def _setup(newton_subs=None):
    so = ctypes.CDLL(ASO)
    ext = types.ModuleType('common.math.external_func')
    ext.so = so
    ext.ctypes = ctypes
    sys.modules['common.math.external_func'] = ext
    sys.path.insert(0, REF)
    m = {
        'common.math.distance': (f'{REF}/common/math/distance.py', []),
        'common.math.math_tools': (f'{REF}/common/math/math_tools.py', []),
        'common.math.ipc': (f'{REF}/common/math/ipc.py', []),
        'common.physics.neo_hookean': (f'{REF}/common/physics/neo_hookean.py', []),
    }
    if newton_subs is not None:
        m['NEWTON_IPC'] = (f'{REF}/projects/FastIPC/NEWTON_IPC.py', newton_subs)
    ti.install(m)
    return so


def V(a):
    return ti.Vector(a)


# ----------------------------------------------------------------------------- unit fixtures
def _contact_quad(rng, scale):
    """Four points whose pairwise features are within ``scale`` (contact-like)."""
    base = rng.uniform(-1, 1, 3)
    pts = base + rng.normal(size=(4, 3)) * scale
    return pts


def gen_unit():
    so = _setup()
    import common.math.distance as D
    import common.math.ipc as I
    import common.math.math_tools as MT
    import common.physics.neo_hookean as NH
    from common.math.graph_tools import find_boundary as ref_find_boundary

    rng = np.random.default_rng(20261203)
    out = {}

    # --- distances and their derivatives (generated closed forms in distance.py)
    N = 64
    pts = np.concatenate([rng.uniform(-1, 1, (N // 2, 4, 3)),
                          np.stack([_contact_quad(rng, 1e-2) for _ in range(N // 2)])])
    out['dist_pts'] = pts
    for name, nv in [('PP_3D', 2), ('PE_3D', 3), ('PT_3D', 4), ('EE_3D', 4), ('EECN2', 4)]:
        Es, gs, Hs = [], [], []
        for q in pts:
            args = [V(q[k]) for k in range(nv)]
            Es.append(getattr(D, name + '_E')(*args))
            gs.append(np.asarray(getattr(D, name + '_g')(*args)).ravel())
            Hs.append(np.asarray(getattr(D, name + '_H')(*args)))
        out[f'{name}_E'] = np.array(Es)
        out[f'{name}_g'] = np.array(gs)
        out[f'{name}_H'] = np.array(Hs)

    # --- types (feature classification) on generic and axis-aligned (tie-prone) inputs
    tpts = np.concatenate([rng.uniform(-1, 1, (256, 4, 3)), rng.integers(-2, 3, (256, 4, 3)).astype(float)])
    out['type_pts'] = tpts
    out['PT_type'] = np.array([D.PT_type(*[V(q[k]) for k in range(4)]) for q in tpts])
    out['EE_type'] = np.array([D.EE_type(*[V(q[k]) for k in range(4)]) for q in tpts])
    out['PE_type'] = np.array([D.PE_type(*[V(q[k]) for k in range(3)]) for q in tpts])

    # --- barrier scalar
    dh2 = 1e-6
    ds = np.concatenate([np.geomspace(1e-14, 1e-6, 40), [1e-6, 2e-6]])
    out['barrier_d'] = ds
    out['barrier_dhat2'] = dh2
    out['barrier_E'] = np.array([D.barrier_E(d, dh2, 1.0) for d in ds])
    out['barrier_g'] = np.array([D.barrier_g(d, dh2, 1.0) for d in ds])
    out['barrier_H'] = np.array([D.barrier_H(d, dh2, 1.0) for d in ds])

    # --- mollifier
    Ms, Mg, MH, thr = [], [], [], []
    mpts = []
    for _ in range(32):
        a0 = rng.uniform(-1, 1, 3)
        a1 = a0 + rng.normal(size=3) * 0.1
        b0 = rng.uniform(-1, 1, 3) * 0.05 + (a0 + a1) / 2
        d = a1 - a0
        b1 = b0 + d * rng.uniform(0.5, 2) + rng.normal(size=3) * 1e-3     # nearly parallel
        q = np.stack([a0, a1, b0, b1])
        mpts.append(q)
        eps = D.M_threshold(*[V(q[k]) for k in range(4)]) * 10.0
        thr.append(eps)
        Ms.append(D.M_E(*[V(q[k]) for k in range(4)], eps))
        Mg.append(np.asarray(D.M_g(*[V(q[k]) for k in range(4)], eps)))
        MH.append(np.asarray(D.M_H(*[V(q[k]) for k in range(4)], eps)))
    out['moll_pts'] = np.array(mpts)
    out['moll_eps'] = np.array(thr)
    out['M_E'], out['M_g'], out['M_H'] = np.array(Ms), np.array(Mg), np.array(MH)

    # --- barrier g and projected H per constraint type (ipc.py *_g_and_H -> a.so project_pd)
    kappa = 3.7e7
    nrow = 24
    for typ in ['PP', 'PE', 'PT', 'EE', 'EEM', 'PPM', 'PEM']:
        X, X0, G, H, E = [], [], [], [], []
        while len(X) < nrow:
            q = _contact_quad(rng, 6e-4)
            q0 = q + rng.normal(size=(4, 3)) * 1e-3
            if typ in ('EEM', 'PPM', 'PEM'):
                # nearly parallel edges: a1-a0 ~ b1-b0
                d = rng.normal(size=3) * 5e-3
                q = np.stack([q[0], q[0] + d, q[2], q[2] + d * 1.1 + rng.normal(size=3) * 1e-6])
                q0 = q.copy()
                q0[1] = q0[0] + d * 3          # rest edges long enough for eps_x > EECN2
                q0[3] = q0[2] + d * 3.1
            vs = [V(q[k]) for k in range(4)]
            v0 = [V(q0[k]) for k in range(4)]
            if typ == 'PP':
                d2 = D.PP_3D_E(vs[0], vs[1])
                if d2 >= dh2:
                    continue
                g, h = I.PP_g_and_H(vs[0], vs[1], dh2, kappa)
                e = I.PP_energy(vs[0], vs[1], dh2, kappa)
            elif typ == 'PE':
                d2 = D.PE_3D_E(vs[0], vs[1], vs[2])
                if d2 >= dh2:
                    continue
                g, h = I.PE_g_and_H(vs[0], vs[1], vs[2], dh2, kappa)
                e = I.PE_energy(vs[0], vs[1], vs[2], dh2, kappa)
            elif typ == 'PT':
                d2 = D.PT_3D_E(*vs)
                if d2 >= dh2:
                    continue
                g, h = I.PT_g_and_H(*vs, dh2, kappa)
                e = I.PT_energy(*vs, dh2, kappa)
            elif typ == 'EE':
                d2 = D.EE_3D_E(*vs)
                if d2 >= dh2:
                    continue
                g, h = I.EE_g_and_H(*vs, dh2, kappa)
                e = I.EE_energy(*vs, dh2, kappa)
            else:
                dist = {'EEM': D.EE_3D_E(*vs), 'PPM': D.PP_3D_E(vs[0], vs[2]),
                        'PEM': D.PE_3D_E(vs[0], vs[2], vs[3])}[typ]
                if dist >= dh2:
                    continue
                if not D.EECN2_E(*vs) < D.M_threshold(*v0):
                    continue
                g, h = getattr(I, typ + '_g_and_H')(*vs, *v0, dh2, kappa)
                e = getattr(I, typ + '_energy')(*vs, *v0, dh2, kappa)
            X.append(q)
            X0.append(q0)
            G.append(np.asarray(g).ravel())
            H.append(np.asarray(h))
            E.append(e)
        out[f'bar_{typ}_x'] = np.array(X)
        out[f'bar_{typ}_x0'] = np.array(X0)
        out[f'bar_{typ}_g'] = np.array(G)
        out[f'bar_{typ}_H'] = np.array(H)
        out[f'bar_{typ}_E'] = np.array(E)
    out['bar_kappa'] = kappa
    out['bar_dhat2'] = dh2

    # --- Neo-Hookean (neo_hookean.py) on deformation gradients near and away from identity
    Fs = np.concatenate([np.eye(3) + rng.normal(size=(16, 3, 3)) * 0.05,
                         np.eye(3) + rng.normal(size=(16, 3, 3)) * 0.3,
                         np.stack([np.eye(3)] * 2)])
    Fs = np.array([F if np.linalg.det(F) > 0.2 else np.eye(3) for F in Fs])
    la, mu = 1e5 * 0.4 / (1.4 * 0.2), 1e5 / 2.8
    out['nh_F'], out['nh_la'], out['nh_mu'] = Fs, la, mu
    ens, Ps, dPs, sig_g, sig_H = [], [], [], [], []
    for F in Fs:
        Fm = ti.Matrix(F)
        U, sig, Vv = ti.svd(Fm)
        ens.append(NH.elasticity_energy(sig, la, mu))
        sig_g.append(np.asarray(NH.elasticity_gradient(sig, la, mu)))
        sig_H.append(np.asarray(NH.elasticity_hessian(sig, la, mu)))
        Ps.append(np.asarray(NH.elasticity_first_piola_kirchoff_stress(Fm, la, mu)))
        dPs.append(np.asarray(NH.elasticity_first_piola_kirchoff_stress_derivative(Fm, la, mu)))
    out['nh_energy'], out['nh_P'], out['nh_dPdF'] = np.array(ens), np.array(Ps), np.array(dPs)
    out['nh_sig_g'], out['nh_sig_H'] = np.array(sig_g), np.array(sig_H)

    # --- 2x2 make_pd (math_tools.py:40-64)
    A2 = rng.normal(size=(64, 2, 2))
    A2 = (A2 + A2.transpose(0, 2, 1)) / 2
    out['mpd_in'] = A2
    out['mpd_out'] = np.array([np.asarray(MT.make_pd(ti.Matrix(a))) for a in A2])

    # --- a.so PSD projection (UTILS.h makePD through wrapper.cpp project_pd_N)
    for n in (3, 6, 9, 12):
        A = rng.normal(size=(16, n, n))
        A = (A + A.transpose(0, 2, 1)) / 2
        res = []
        for a in A:
            outs = ti.ext_call(getattr(so, f'project_pd_{n}'), tuple(a.ravel()), n * n)
            res.append(np.array(outs).reshape(n, n))
        out[f'ppd{n}_in'], out[f'ppd{n}_out'] = A, np.array(res)

    # --- a.so svd_3 (JGSL)
    Fsv = np.concatenate([rng.normal(size=(16, 3, 3)), Fs[:8]])
    svd_out = []
    for F in Fsv:
        o = np.array(ti.ext_call(so.svd_3, tuple(F.ravel()), 27))
        svd_out.append(o)
    out['svd_in'], out['svd_out'] = Fsv, np.array(svd_out)

    # --- tet inversion-free step (math_tools.py:161-181 -> a.so cubic root)
    cub_x, cub_p, cub_t = [], [], []
    for _ in range(128):
        xs = np.eye(4, 3) * 0 + rng.normal(size=(4, 3)) * 0.01
        xs[1:] += np.eye(3) * 0.02
        ps = rng.normal(size=(4, 3)) * 0.02
        t = MT.get_smallest_positive_real_cubic_root(*[V(a) for a in xs], *[V(a) for a in ps], 0.2)
        cub_x.append(xs)
        cub_p.append(ps)
        cub_t.append(t)
    out['cubic_x'], out['cubic_p'], out['cubic_t'] = np.array(cub_x), np.array(cub_p), np.array(cub_t)

    # --- CCD (ipc.py point_triangle_ccd / edge_edge_ccd -> a.so EVCTCD), eta = 0.2
    for kind in ('pt', 'ee'):
        Xs, Ps_, Ts = [], [], []
        for it in range(192):
            x = _contact_quad(rng, 2e-3)
            p = rng.normal(size=(4, 3)) * 10 ** rng.uniform(-4, -1.5)
            if it % 3 == 0:   # drive the first primitive through the second
                p[0] = (x[1:].mean(0) - x[0]) * rng.uniform(0.5, 3) + rng.normal(size=3) * 1e-4
            vs = [V(a) for a in x]
            ds = [V(a) for a in p]
            if kind == 'pt':
                dist2 = D.PT_dist2(*vs, D.PT_type(*vs))
                toc = I.point_triangle_ccd(*vs, *ds, 0.2, dist2)
            else:
                dist2 = D.EE_dist2(*vs, D.EE_type(*vs))
                toc = I.edge_edge_ccd(*vs, *ds, 0.2, dist2)
            Xs.append(x)
            Ps_.append(p)
            Ts.append(toc)
        out[f'ccd_{kind}_x'], out[f'ccd_{kind}_p'], out[f'ccd_{kind}_toc'] = np.array(Xs), np.array(Ps_), np.array(Ts)

    # --- segment/triangle intersection (ipc.py:511-526)
    seg = rng.normal(size=(256, 5, 3))
    out['seg_pts'] = seg
    out['seg_hit'] = np.array([bool(I.segment_intersect_triangle(*[V(a) for a in s])) for s in seg])

    # --- find_boundary (graph_tools.py) on the reference cube pattern
    from fastipc_gb300 import scenes
    _, tets = scenes.hex_grid(3, 3, 3)
    bp, be, bt = ref_find_boundary(tets)
    out['fb_tets'] = tets
    out['fb_points'] = np.array(sorted(bp))
    out['fb_edges'] = np.asarray(be)
    out['fb_tris'] = np.asarray(bt)

    np.savez_compressed(os.path.join(HERE, 'unit_kernels.npz'), **out)
    print('wrote unit_kernels.npz', len(out), 'arrays')


# ----------------------------------------------------------------------------- reference cube mesh
def gen_cube_mesh():
    """reader.py add_object('cube') (n = 10 vertices per side) executed from its source."""
    src = open(f'{REF}/projects/FastIPC/reader.py').read()
    start = src.index("    if filename == 'cube':")
    end = src.index("    elif filename[-4:] == '.msh':")
    body = src[start:end].replace("    if filename == 'cube':", "if True:")
    body = '\n'.join(line[4:] if line.startswith('    ') else line for line in body.split('\n'))
    ns = {'np': np}
    exec(body, ns)
    np.savez_compressed(os.path.join(HERE, 'cube_mesh.npz'), particles=ns['new_particles'], elements=ns['new_elements'])
    print('wrote cube_mesh.npz')


# ----------------------------------------------------------------------------- reference Newton run
def gen_newton(n=3, steps=6, seed=0, record_iters=11, matrix_iters=(0, 2, 5)):
    """Run NEWTON_IPC.py's own functions on a small two-cube scene and record every step.

    The scene starts pre-deformed by +-0.5 mm (scenes.predeform).
    Source edits (the same ones the CPU-baseline notes list): Neo-Hookean import instead of
    fixed-corotated, dt = 0.01, E = 1e5, nu = 0.4, smaller MAX_LINEAR/MAX_C buffers.
    d-hat^2 stays 1e-6 (d-hat = 1e-3 m, as in the two-cube scene).  The driver loop below
    follows NEWTON_IPC.py:955-996 statement by statement, calling the module's functions.
    """
    from fastipc_gb300 import scenes
    scene = scenes.predeform(scenes.two_cubes(n=n, seed=seed), 5e-4, seed)
    subs = [
        ('from common.physics.fixed_corotated import *', 'from common.physics.neo_hookean import *'),
        ('dt = 0.04', 'dt = 0.01'),
        ('MAX_LINEAR = 50000000 if dim == 3 else 5000000', 'MAX_LINEAR = 400000'),
        ('MAX_C = 100000', 'MAX_C = 20000'),
        ('        E = 2.e4\n    nu = 0.4', '        E = 1.e5\n    nu = 0.4'),
    ]
    _setup(subs)
    import scipy.sparse
    import scipy.sparse.linalg as spla

    reader = types.ModuleType('reader')
    settings = {
        'mesh_particles': scene.x.copy(), 'mesh_elements': scene.tets.copy(), 'dim': 3,
        'gravity': scene.gravity, 'start_frame': 0,
        'boundary': (set(scene.boundary_points.tolist()), scene.boundary_edges.copy(), scene.boundary_triangles.copy()),
        'dirichlet': scene.dirichlet, 'mesh_scale': 1.0, 'mesh_offset': [0., 0., 0.],
    }
    reader.read = lambda: settings
    reader.np = np
    sys.modules['reader'] = reader
    sys.modules['meshio'] = types.ModuleType('meshio')
    chol = types.ModuleType('sksparse.cholmod')

    def cholesky(A):
        lu = spla.splu(A.tocsc())
        return lambda b: lu.solve(b)
    chol.cholesky = cholesky
    sys.modules['sksparse'] = types.ModuleType('sksparse')
    sys.modules['sksparse.cholmod'] = chol
    os.chdir(tempfile.mkdtemp(prefix='fastipc_golden_'))
    sys.argv = ['NEWTON_IPC.py', '1008', '0']
    import NEWTON_IPC as R

    # boundary order exactly as the scene lists it (the reference converts the point set)
    R.x.from_numpy(scene.x.astype(np.float64))
    R.v.fill(0)
    R.v.from_numpy(scene.v.astype(np.float64))
    R.vertices.from_numpy(scene.tets.astype(np.int32))
    R.boundary_points.from_numpy(scene.boundary_points.astype(np.int32))
    R.boundary_edges.from_numpy(scene.boundary_edges.astype(np.int32))
    R.boundary_triangles.from_numpy(scene.boundary_triangles.astype(np.int32))
    R.compute_restT_and_m()
    R.kappa = R.compute_adaptive_kappa() * 10
    R.spatial_hash_inv_dx = 1.0 / R.compute_mean_of_boundary_edges()
    R.save_x0()
    # start from the pre-deformed state (rest shape, x0, kappa and the hash cell keep the
    # rest positions); see scenes.predeform for why
    R.x.from_numpy(scene.initial_positions().astype(np.float64))
    rec = {'x_init': scene.initial_positions(), 'x_rest': scene.x, 'predeform': 5e-4, 'v_init': scene.v, 'tets': scene.tets,
           'bpoints': scene.boundary_points, 'bedges': scene.boundary_edges, 'btris': scene.boundary_triangles,
           'kappa': R.kappa, 'inv_dx': R.spatial_hash_inv_dx, 'mass': R.m.to_numpy(),
           'dt': R.dt, 'dhat2': R.dHat2, 'n': n, 'seed': seed, 'steps': steps}
    names = ['PP', 'PE', 'PT', 'EE', 'EEM', 'PPM', 'PEM']
    xs, vs, iters = [], [], []
    it_global = 0
    for f in range(steps):
        R.compute_xn_and_xTilde()
        R.move_nodes(f * R.dt)
        newton_iter = 0
        while True:
            newton_iter += 1
            R.find_constraints()
            R.data_row.fill(0)
            R.data_col.fill(0)
            R.data_val.fill(0)
            R.data_rhs.fill(0)
            R.data_sol.fill(0)
            R.compute_hessian_and_gradient()
            if it_global < record_iters:
                k = f'it{it_global}_'
                rec[k + 'x'] = R.x.to_numpy()
                rec[k + 'xtilde'] = R.xTilde.to_numpy()
                for nm in names:
                    cnt = getattr(R, 'n_' + nm)[None]
                    rec[k + nm] = getattr(R, nm).to_numpy()[:cnt]
                c = R.cnt[None]
                if it_global in matrix_iters:
                    # the system matrix before the Dirichlet edit, duplicates summed (CSR)
                    nd = 3 * len(scene.x)
                    A = scipy.sparse.csr_matrix((R.data_val.to_numpy()[:c], (R.data_row.to_numpy()[:c],
                                                 R.data_col.to_numpy()[:c])), shape=(nd, nd))
                    A.sort_indices()
                    rec[k + 'A_data'], rec[k + 'A_indices'], rec[k + 'A_indptr'] = A.data, A.indices, A.indptr
                rec[k + 'rhs'] = R.data_rhs.to_numpy()
            R.solve_system(f * R.dt)
            res = R.output_residual()
            if it_global < record_iters:
                rec[k + 'sol'] = R.data_sol.to_numpy()
                rec[k + 'residual'] = res
            if res < 1e-2 * R.dt:
                it_global += 1
                break
            E0 = R.compute_energy()
            R.save_xPrev()
            alpha = R.compute_intersection_free_step_size()
            alpha_ccd = alpha
            R.apply_sol(alpha)
            while R.check_collision():
                alpha /= 2.0
                R.apply_sol(alpha)
            R.find_constraints()
            E = R.compute_energy()
            while E > E0:
                alpha *= 0.5
                R.apply_sol(alpha)
                R.find_constraints()
                E = R.compute_energy()
            while R.check_collision():
                alpha /= 2.0
                R.apply_sol(alpha)
            if it_global < record_iters:
                rec[k + 'E0'] = E0
                rec[k + 'alpha_ccd'] = alpha_ccd
                rec[k + 'alpha'] = alpha
                rec[k + 'E'] = E
                rec[k + 'x_after'] = R.x.to_numpy()
            it_global += 1
            print(f'  step {f} newton {newton_iter} res {res:.3e} alpha {alpha:.4f}', flush=True)
        R.compute_v()
        xs.append(R.x.to_numpy())
        vs.append(R.v.to_numpy())
        iters.append(newton_iter)
        print(f'step {f}: {newton_iter} newton iterations', flush=True)
    rec['x_steps'] = np.array(xs)
    rec['v_steps'] = np.array(vs)
    rec['newton_iters'] = np.array(iters)
    np.savez_compressed(os.path.join(HERE, f'newton_two_cubes_n{n}.npz'), **rec)
    print('wrote', f'newton_two_cubes_n{n}.npz')


def gen_newton2d(n=3, steps=6, seed=0, record_iters=12):
    """Run NEWTON_IPC.py's own functions with dim == 2 (fixed-corotated triangles, the
    reference's default material) on a small two-square scene with a fixed ground segment and
    record every step and every Newton iteration.

    Source edits: dt = 0.01, E = 1e5, smaller MAX_LINEAR/MAX_C buffers, no GUI window.  d-hat^2
    stays 1e-6.
    The loop follows NEWTON_IPC.py:955-996 statement by statement.
    """
    from fastipc_gb300 import scenes
    # pre-deformed start, as for the 3D fixture: at an exactly undeformed triangle the projected
    # twist block of the reference's dP/dF depends on the sign of rounding noise
    scene = scenes.predeform(scenes.two_squares_2d(n=n, seed=seed), 5e-4, seed)
    subs = [
        ('dt = 0.04', 'dt = 0.01'),
        ('MAX_LINEAR = 50000000 if dim == 3 else 5000000', 'MAX_LINEAR = 100000'),
        ('MAX_C = 100000', 'MAX_C = 5000'),
        ('        E = 2.e4\n    nu = 0.4', '        E = 1.e5\n    nu = 0.4'),
        # the 2D GUI window (images of write_image) is not part of the path: not created
        ('    gui = ti.GUI("IPC", (768, 768), background_color=0x112F41)', '    gui = None'),
    ]
    _setup(subs)
    import scipy.sparse.linalg as spla

    reader = types.ModuleType('reader')
    settings = {
        'mesh_particles': scene.x.copy(), 'mesh_elements': scene.tris.copy(), 'dim': 2,
        'gravity': scene.gravity, 'start_frame': 0,
        'boundary': (set(scene.boundary_points.tolist()), scene.boundary_edges.copy(), np.array([[-1, -1, -1]])),
        'dirichlet': scene.dirichlet, 'mesh_scale': 1.0, 'mesh_offset': [0., 0.],
    }
    reader.read = lambda: settings
    reader.np = np
    sys.modules['reader'] = reader
    sys.modules['meshio'] = types.ModuleType('meshio')
    chol = types.ModuleType('sksparse.cholmod')

    def cholesky(A):
        lu = spla.splu(A.tocsc())
        return lambda b: lu.solve(b)
    chol.cholesky = cholesky
    sys.modules['sksparse'] = types.ModuleType('sksparse')
    sys.modules['sksparse.cholmod'] = chol
    os.chdir(tempfile.mkdtemp(prefix='fastipc_golden2d_'))
    sys.argv = ['NEWTON_IPC.py', '2', '0']
    import NEWTON_IPC as R

    R.x.from_numpy(scene.x.astype(np.float64))
    R.v.fill(0)
    R.v.from_numpy(scene.v.astype(np.float64))
    R.vertices.from_numpy(scene.tris.astype(np.int32))
    R.boundary_points.from_numpy(scene.boundary_points.astype(np.int32))
    R.boundary_edges.from_numpy(scene.boundary_edges.astype(np.int32))
    R.compute_restT_and_m()
    R.kappa = R.compute_adaptive_kappa() * 10
    R.spatial_hash_inv_dx = 1.0 / R.compute_mean_of_boundary_edges()
    R.save_x0()
    R.x.from_numpy(scene.initial_positions().astype(np.float64))
    rec = {'x_rest': scene.x, 'x_init': scene.initial_positions(), 'predeform': 5e-4, 'v_init': scene.v, 'tris': scene.tris, 'bpoints': scene.boundary_points,
           'bedges': scene.boundary_edges, 'kappa': R.kappa, 'mean_edge': 1.0 / R.spatial_hash_inv_dx, 'mass': R.m.to_numpy(),
           'dt': R.dt, 'dhat2': R.dHat2, 'n': n, 'seed': seed, 'steps': steps}
    # the reference's own boundary extraction (graph_tools.py:8-25) on the scenes' triangles
    from common.math.graph_tools import find_boundary as ref_find_boundary
    rbp, rbe, _ = ref_find_boundary(scene.tris)
    rec['ref_bpoints'], rec['ref_bedges'] = np.array(sorted(rbp)), np.asarray(rbe)
    stack = scenes.square_stack_2d(k=3, n=4, seed=1)
    rbp, rbe, _ = ref_find_boundary(stack.tris)
    rec['stack_tris'], rec['stack_ref_bpoints'], rec['stack_ref_bedges'] = stack.tris, np.array(sorted(rbp)), np.asarray(rbe)
    xs, vs, iters = [], [], []
    it_global = 0
    nd = 2 * len(scene.x)
    for f in range(steps):
        R.compute_xn_and_xTilde()
        R.move_nodes(f * R.dt)
        newton_iter = 0
        while True:
            newton_iter += 1
            R.find_constraints()
            R.data_row.fill(0)
            R.data_col.fill(0)
            R.data_val.fill(0)
            R.data_rhs.fill(0)
            R.data_sol.fill(0)
            R.compute_hessian_and_gradient()
            # the first record_iters iterations under it{i}_ (every consumer), the rest under xt{i}_
            # with '_res' for the residual (oracle tests only)
            k = f'it{it_global}_' if it_global < record_iters else f'xt{it_global}_'
            rec[k + 'x'] = R.x.to_numpy()
            rec[k + 'xtilde'] = R.xTilde.to_numpy()
            rec[k + 'PP'] = R.PP.to_numpy()[:R.n_PP[None]]
            rec[k + 'PE'] = R.PE.to_numpy()[:R.n_PE[None]]
            c = R.cnt[None]
            import scipy.sparse
            A = scipy.sparse.csr_matrix((R.data_val.to_numpy()[:c], (R.data_row.to_numpy()[:c], R.data_col.to_numpy()[:c])),
                                        shape=(nd, nd))
            A.sort_indices()
            rec[k + 'A_data'], rec[k + 'A_indices'], rec[k + 'A_indptr'] = A.data, A.indices, A.indptr
            rec[k + 'rhs'] = R.data_rhs.to_numpy()
            R.solve_system(f * R.dt)
            res = R.output_residual()
            rec[k + 'sol'] = R.data_sol.to_numpy()
            rec[k + ('residual' if it_global < record_iters else 'res')] = res
            if res < 1e-2 * R.dt:
                it_global += 1
                break
            E0 = R.compute_energy()
            R.save_xPrev()
            alpha = R.compute_intersection_free_step_size()
            alpha_ccd = alpha
            R.apply_sol(alpha)
            while R.check_collision():
                alpha /= 2.0
                R.apply_sol(alpha)
            R.find_constraints()
            E = R.compute_energy()
            while E > E0:
                alpha *= 0.5
                R.apply_sol(alpha)
                R.find_constraints()
                E = R.compute_energy()
            while R.check_collision():
                alpha /= 2.0
                R.apply_sol(alpha)
            rec[k + 'E0'] = E0
            rec[k + 'alpha_ccd'] = alpha_ccd
            rec[k + 'alpha'] = alpha
            rec[k + 'E'] = E
            it_global += 1
            print(f'  step {f} newton {newton_iter} res {res:.3e} alpha {alpha:.4f}', flush=True)
        R.compute_v()
        xs.append(R.x.to_numpy())
        vs.append(R.v.to_numpy())
        iters.append(newton_iter)
        print(f'step {f}: {newton_iter} newton iterations', flush=True)
    rec['x_steps'] = np.array(xs)
    rec['v_steps'] = np.array(vs)
    rec['newton_iters'] = np.array(iters)
    np.savez_compressed(os.path.join(HERE, f'newton2d_two_squares_n{n}.npz'), **rec)
    print('wrote', f'newton2d_two_squares_n{n}.npz')


if __name__ == '__main__':
    what = sys.argv[1] if len(sys.argv) > 1 else 'all'
    if what in ('unit', 'all'):
        gen_cube_mesh()
        gen_unit()
    if what in ('newton', 'all'):
        gen_newton()
    if what in ('newton2d', 'all'):
        gen_newton2d()
