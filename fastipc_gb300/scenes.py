"""Synthetic scenes for the IPC Newton path (numpy, set-up only).

A scene is a tet mesh plus its surface (boundary points, oriented boundary edges p0 < p1,
outward boundary triangles) and a Dirichlet schedule ``dirichlet(t) -> (mask[V], target[V,3])``,
i.e. the ``settings`` dict that ``projects/FastIPC/reader.py:read()`` returns.

Meshes are hexahedral grids split into 6 tets per hex with the split pattern of the
reference's ``cube`` generator (``projects/FastIPC/reader.py:37-63``): vertex (i, j, k) of an
(nx+1)x(ny+1)x(nz+1) grid has index ``i*(ny+1)*(nz+1) + j*(nz+1) + k`` and hex corner list
``f = [000, 100, 101, 001, 010, 110, 111, 011]`` (i, j, k offsets) produces the tets
``[f0 f4 f6 f5] [f3 f6 f2 f0] [f0 f4 f7 f6] [f3 f6 f0 f7] [f2 f0 f6 f1] [f6 f0 f5 f1]``.
The pattern has to match because it fixes the tet orientation and the surface triangulation.
"""
from dataclasses import dataclass, field
from typing import Callable

import numpy as np

# hex corner (di, dj, dk) for f0..f7 and the six tets of one hex (reader.py:50-63)
_HEX_CORNERS = np.array([[0, 0, 0], [1, 0, 0], [1, 0, 1], [0, 0, 1],
                         [0, 1, 0], [1, 1, 0], [1, 1, 1], [0, 1, 1]], dtype=np.int64)
_HEX_TETS = np.array([[0, 4, 6, 5], [3, 6, 2, 0], [0, 4, 7, 6],
                      [3, 6, 0, 7], [2, 0, 6, 1], [6, 0, 5, 1]], dtype=np.int64)


def hex_grid(nx, ny, nz, size=(1.0, 1.0, 1.0)):
    """Vertices [V,3] f64 and tets [6*nx*ny*nz, 4] i32 of an axis-aligned box [0,size]."""
    Nx, Ny, Nz = nx + 1, ny + 1, nz + 1
    i, j, k = np.meshgrid(np.arange(Nx), np.arange(Ny), np.arange(Nz), indexing='ij')
    verts = np.stack([i.ravel() * (size[0] / nx), j.ravel() * (size[1] / ny),
                      k.ravel() * (size[2] / nz)], axis=1).astype(np.float64)
    hi, hj, hk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing='ij')
    base = np.stack([hi.ravel(), hj.ravel(), hk.ravel()], axis=1)          # hex order i, j, k
    corner = base[:, None, :] + _HEX_CORNERS[None, :, :]                     # [H, 8, 3]
    f = corner[..., 0] * (Ny * Nz) + corner[..., 1] * Nz + corner[..., 2]    # [H, 8]
    tets = f[:, _HEX_TETS].reshape(-1, 4)                                    # [H*6, 4]
    return verts, tets.astype(np.int32)


def find_boundary(tets):
    """Surface of a tet mesh, ``common/math/graph_tools.py:26-45`` semantics.

    Each tet contributes the faces (p0,p2,p1) (p0,p3,p2) (p0,p1,p3) (p1,p2,p3); a face is on
    the boundary when no face with the opposite orientation exists.  Boundary triangles keep
    the tet's face orientation; an edge p->q of a boundary triangle is kept when p < q (each
    surface edge exactly once); the points are the vertices of boundary triangles.

    The reference iterates a python set, so its list order is hash order; here triangles come
    in (tet, face) order, edges in the order they first appear from the triangles and points
    ascending.  Only the edge order is observable downstream (edge-edge pairs are taken as
    (lower list index, higher list index)).
    """
    tets = np.asarray(tets, dtype=np.int64)
    faces = np.concatenate([tets[:, [0, 2, 1]], tets[:, [0, 3, 2]],
                            tets[:, [0, 1, 3]], tets[:, [1, 2, 3]]], axis=0)
    order = np.arange(len(faces)).reshape(4, -1).T.ravel()                  # (tet, face) order
    faces = faces[order]
    key = np.sort(faces, axis=1)
    _, inv, cnt = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    tris = faces[cnt[inv.ravel()] == 1]
    e = np.stack([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]], axis=1).reshape(-1, 2)
    edges = e[e[:, 0] < e[:, 1]]
    points = np.unique(tris.ravel())
    return points.astype(np.int32), edges.astype(np.int32), tris.astype(np.int32)


def rotation_matrix(axis, angle):
    """Rodrigues rotation about unit ``axis`` by ``angle`` radians."""
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * (K @ K)


@dataclass
class Scene:
    name: str
    x: np.ndarray                 # [V,3] f64 rest/initial positions
    tets: np.ndarray              # [T,4] i32
    v: np.ndarray                 # [V,3] f64 initial velocity
    boundary_points: np.ndarray   # [Vs] i32
    boundary_edges: np.ndarray    # [Es,2] i32
    boundary_triangles: np.ndarray  # [Fs,3] i32
    dirichlet: Callable           # t -> (mask[V] bool, target[V,3] f64)
    E: float = 1e5
    nu: float = 0.4
    rho: float = 1000.0
    dhat: float = 1e-3
    dt: float = 0.01
    gravity: float = -9.8
    steps: int = 50
    meta: dict = field(default_factory=dict)
    x_init: np.ndarray = None     # [V,3] initial positions when they differ from the rest shape
    # the Dirichlet schedule as rigid motions of vertex groups, evaluated on the device by
    # fipc_dirichlet_script when present: group [V] i32 (-1 free), motion [G,10] f64 =
    # (centre[3], unit axis[3], omega rad/s, velocity[3]); ``dirichlet`` is the same schedule
    # written as the reference's per-vertex loop
    dirichlet_groups: np.ndarray = None
    dirichlet_motion: np.ndarray = None

    def initial_positions(self):
        return self.x if self.x_init is None else self.x_init

    @property
    def n_verts(self):
        return len(self.x)

    @property
    def n_tets(self):
        return len(self.tets)


def _finish(name, parts, v, dirichlet_fn, script=None, **kw):
    xs, ts, off = [], [], 0
    for x, t in parts:
        xs.append(x)
        ts.append(t + off)
        off += len(x)
    x = np.concatenate(xs).astype(np.float64)
    tets = np.concatenate(ts).astype(np.int32)
    bp, be, bt = find_boundary(tets)
    groups, motion = (None, None) if script is None else script
    return Scene(name, x, tets, v, bp, be, bt, dirichlet_fn(x), dirichlet_groups=groups, dirichlet_motion=motion, **kw)


def motion_row(centre=(0.0, 0.0, 0.0), axis=(1.0, 0.0, 0.0), omega=0.0, velocity=(0.0, 0.0, 0.0)):
    """One group's rigid motion for fipc_dirichlet_script: rotation about the unit ``axis``
    through ``centre`` at ``omega`` rad/s, then translation at ``velocity``."""
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    return np.concatenate([np.asarray(centre, dtype=np.float64), a, [float(omega)], np.asarray(velocity, dtype=np.float64)])


def _static_dirichlet(mask):
    def make(x):
        x_rest = x.copy()
        return lambda t: (mask, x_rest)
    return make


def _static_script(mask):
    """A fixed mask as one motionless group: targets equal the rest positions exactly."""
    return np.where(mask, 0, -1).astype(np.int32), motion_row()[None, :]


def two_cubes(n=8, seed=0, side=0.1, gap=2e-3, max_angle_deg=15.0, speed=1.0, E=1e5, nu=0.4, steps=50):
    """Lower cube with its bottom face fixed; upper cube rotated by a seed-drawn angle
    (<= max_angle_deg about a seed-drawn axis) whose lowest vertex sits ``gap`` above the
    lower cube's top face, moving at ``-speed`` m/s along y."""
    rng = np.random.default_rng(seed)
    lo, lt = hex_grid(n, n, n, (side, side, side))
    up, ut = hex_grid(n, n, n, (side, side, side))
    axis = rng.normal(size=3)
    angle = np.deg2rad(rng.uniform(0.0, max_angle_deg))
    R = rotation_matrix(axis, angle)
    c = np.full(3, side / 2)
    up = (up - c) @ R.T + c
    up[:, 1] += side + gap - up[:, 1].min()
    nv = len(lo) + len(up)
    v = np.zeros((nv, 3))
    v[len(lo):, 1] = -speed
    mask = np.zeros(nv, dtype=bool)
    mask[:len(lo)] = lo[:, 1] <= 1e-12
    return _finish('two_cubes', [(lo, lt), (up, ut)], v, _static_dirichlet(mask), script=_static_script(mask), E=E, nu=nu,
                   steps=steps,
                   meta={'seed': seed, 'n': n, 'axis': axis.tolist(), 'angle': float(angle)})


def cube_lattice(m=6, n=6, seed=0, side=0.1, gap=2e-3, jitter=0.1, ground=(2.0, 0.1, 2.0), steps=100):
    """m^3 cubes (n hexes per side) with seed-drawn rotations and +-jitter*side position
    jitter, dropped under gravity onto a fixed ground box; every cube's bounding sphere keeps
    at least ``gap`` to its neighbours and to the ground."""
    rng = np.random.default_rng(seed)
    base_x, base_t = hex_grid(n, n, n, (side, side, side))
    r = np.sqrt(3) * side / 2                           # bounding-sphere radius
    pitch = 2 * r + gap + 2 * jitter * side
    parts = []
    gx, gy, gz = ground
    gnd_x, gnd_t = hex_grid(1, 1, 1, (gx, gy, gz))
    gnd_x = gnd_x + np.array([-gx / 2, -gy, -gz / 2])
    for a in range(m):
        for b in range(m):
            for c in range(m):
                R = rotation_matrix(rng.normal(size=3), rng.uniform(0, 2 * np.pi))
                ctr = np.array([(a - (m - 1) / 2) * pitch, r + gap + b * pitch, (c - (m - 1) / 2) * pitch])
                ctr += rng.uniform(-jitter, jitter, 3) * side
                ctr[1] = max(ctr[1], r + gap)
                parts.append(((base_x - side / 2) @ R.T + ctr, base_t))
    parts.append((gnd_x, gnd_t))
    nv = sum(len(p[0]) for p in parts)
    mask = np.zeros(nv, dtype=bool)
    mask[nv - len(gnd_x):] = True
    return _finish('cube_lattice', parts, np.zeros((nv, 3)), _static_dirichlet(mask), script=_static_script(mask), steps=steps,
                   meta={'seed': seed, 'm': m, 'n': n})


def twisted_bar(nx=400, ny=20, nz=20, size=(1.0, 0.05, 0.05), seed=0, jitter=1e-4, speed=np.pi,
                E=1e6, nu=0.45, dhat=5e-4, steps=200):
    """Bar along x centred at the origin; both end faces are Dirichlet and rotate about the
    x axis, the x<0 end at +speed and the x>0 end at -speed rad/s, in the form of the
    reference's mat-twist schedule (``projects/FastIPC/reader.py:170-185``).  All vertices get
    seed-drawn uniform +-jitter at t=0."""
    rng = np.random.default_rng(seed)
    x, t = hex_grid(nx, ny, nz, size)
    x -= np.array(size) / 2
    ends = (np.abs(x[:, 0]) >= size[0] / 2 - 1e-12)
    x = x + rng.uniform(-jitter, jitter, x.shape)

    def make(x0):
        x_rest = x0.copy()
        a, b, c = x_rest[:, 0], x_rest[:, 1], x_rest[:, 2]
        radius = np.sqrt(b * b + c * c)
        ang0 = np.arctan2(b, c)
        sgn = np.where(a < 0, 1.0, -1.0)

        def dirichlet(tm):
            target = x_rest.copy()
            ang = ang0 + speed * tm * sgn
            target[ends, 1] = (radius * np.sin(ang))[ends]
            target[ends, 2] = (radius * np.cos(ang))[ends]
            return ends, target
        return dirichlet

    # the same schedule as rigid motions: the x<0 end turns about +x at -speed (its angle
    # atan2(y, z) grows), the x>0 end at +speed
    groups = np.where(ends, np.where(x[:, 0] < 0, 0, 1), -1).astype(np.int32)
    motion = np.stack([motion_row(omega=-speed), motion_row(omega=speed)])
    return _finish('twisted_bar', [(x, t)], np.zeros_like(x), make, script=(groups, motion), E=E, nu=nu, dhat=dhat,
                   gravity=0.0, steps=steps, meta={'seed': seed, 'nx': nx, 'ny': ny, 'nz': nz})


def predeform(scene, amplitude, seed=0):
    """Start ``scene`` from its rest shape plus seeded uniform +-amplitude displacements on
    the free vertices.  At an exactly undeformed element the reference's projected
    Neo-Hookean Hessian depends on the sign of rounding noise (its 2x2 make_pd acts on the
    twist/flip blocks only when a coefficient is negative), so states used for
    iteration-by-iteration parity start away from rest."""
    rng = np.random.default_rng(seed + 7919)
    mask, _ = scene.dirichlet(0.0)
    d = rng.uniform(-amplitude, amplitude, scene.x.shape)
    d[mask] = 0.0
    scene.x_init = scene.x + d
    scene.meta['predeform'] = amplitude
    return scene


def cube_stack(seed, side=0.1, gap=2e-3, min_cubes=1, max_cubes=8, min_hex=3, max_hex=10, ground=(1.0, 0.1, 1.0),
               jitter=0.1, steps=50):
    """A seed-drawn stack of 1-8 cubes, each with a seed-drawn 3-10 hexes per side, randomly
    rotated and stacked along y with at least ``gap`` between bounding spheres, above a fixed
    ground box; horizontal centres get +-jitter*side.  Sizes run from 168 to 48,006 tets."""
    rng = np.random.default_rng(seed)
    k = int(rng.integers(min_cubes, max_cubes + 1))
    r = np.sqrt(3) * side / 2
    parts = []
    y = gap + r
    for _ in range(k):
        n = int(rng.integers(min_hex, max_hex + 1))
        bx, bt = hex_grid(n, n, n, (side, side, side))
        R = rotation_matrix(rng.normal(size=3), rng.uniform(0, 2 * np.pi))
        ctr = np.array([rng.uniform(-jitter, jitter) * side, y, rng.uniform(-jitter, jitter) * side])
        parts.append(((bx - side / 2) @ R.T + ctr, bt))
        y += 2 * r + gap
    gx, gy, gz = ground
    gnd_x, gnd_t = hex_grid(1, 1, 1, (gx, gy, gz))
    parts.append((gnd_x + np.array([-gx / 2, -gy, -gz / 2]), gnd_t))
    nv = sum(len(p[0]) for p in parts)
    mask = np.zeros(nv, dtype=bool)
    mask[nv - len(gnd_x):] = True
    return _finish('cube_stack', parts, np.zeros((nv, 3)), _static_dirichlet(mask), script=_static_script(mask), steps=steps,
                   meta={'seed': seed, 'cubes': k})


def cube_stacks(n_scenes=512, seed=0, **kw):
    """``n_scenes`` independent cube stacks with seeds seed, seed+1, ...: the batched workload."""
    return [cube_stack(seed + i, **kw) for i in range(n_scenes)]


# ------------------------------------------------------------------------------ 2D scenes
def tri_grid(nx, ny, size=(1.0, 1.0)):
    """Vertices [V,2] f64 and counter-clockwise triangles [2*nx*ny, 3] i32 of the box
    [0,size]: every quad split along its (i,j)-(i+1,j+1) diagonal."""
    Nx, Ny = nx + 1, ny + 1
    i, j = np.meshgrid(np.arange(Nx), np.arange(Ny), indexing='ij')
    verts = np.stack([i.ravel() * (size[0] / nx), j.ravel() * (size[1] / ny)], axis=1).astype(np.float64)
    qi, qj = np.meshgrid(np.arange(nx), np.arange(ny), indexing='ij')
    a = (qi * Ny + qj).ravel()
    b, c, d = a + Ny, a + Ny + 1, a + 1                    # (i+1,j), (i+1,j+1), (i,j+1)
    tris = np.concatenate([np.stack([a, b, c], 1), np.stack([a, c, d], 1)], axis=1).reshape(-1, 3)
    return verts, tris.astype(np.int32)


def find_boundary_2d(tris):
    """find_boundary of common/math/graph_tools.py:8-25 for triangles: a half-edge (i, j) without
    its twin (j, i) gives the boundary edge [j, i], in triangle order."""
    edges = set()
    for i, j, k in tris.tolist():
        edges.update([(i, j), (j, k), (k, i)])
    pts, be = set(), []
    for i, j, k in tris.tolist():
        for a, b in ((i, j), (j, k), (k, i)):
            if (b, a) not in edges:
                pts.update([b, a])
                be.append([b, a])
    return np.array(sorted(pts), dtype=np.int32), np.array(be, dtype=np.int32).reshape(-1, 2)


@dataclass
class Scene2D:
    name: str
    x: np.ndarray                 # [V,2] f64 rest/initial positions
    tris: np.ndarray              # [T,3] i32
    v: np.ndarray                 # [V,2] f64 initial velocity
    boundary_points: np.ndarray   # [Vs] i32
    boundary_edges: np.ndarray    # [Es,2] i32
    dirichlet: Callable           # t -> (mask[V] bool, target[V,2] f64)
    E: float = 1e5
    nu: float = 0.4
    rho: float = 1000.0
    dhat: float = 1e-3
    dt: float = 0.01
    gravity: float = -9.8
    steps: int = 50
    meta: dict = field(default_factory=dict)
    x_init: np.ndarray = None

    def initial_positions(self):
        return self.x if self.x_init is None else self.x_init

    @property
    def n_verts(self):
        return len(self.x)


def _rot2(a):
    return np.array([[np.cos(a), -np.sin(a)], [np.sin(a), np.cos(a)]])


def two_squares_2d(n=4, seed=0, side=0.1, gap=2e-3, max_angle_deg=15.0, speed=1.0, E=1e5, nu=0.4, segment=True, steps=50):
    """The 2D counterpart of ``two_cubes``: a lower square whose bottom row is fixed and an
    upper square rotated by a seed-drawn angle (<= max_angle_deg), its lowest vertex ``gap``
    above the lower one, moving at -speed m/s along y.  With ``segment``, a fixed ground
    segment below the lower square is added as two boundary points and one boundary edge
    without elements, as the reference's add_boundary does (projects/FastIPC/reader.py:87-101)."""
    rng = np.random.default_rng(seed)
    lo, lt = tri_grid(n, n, (side, side))
    up, ut = tri_grid(n, n, (side, side))
    ang = np.deg2rad(rng.uniform(-max_angle_deg, max_angle_deg))
    c = np.full(2, side / 2)
    up = (up - c) @ _rot2(ang).T + c
    up[:, 1] += side + gap - up[:, 1].min()
    x = np.concatenate([lo, up])
    tris = np.concatenate([lt, ut + len(lo)]).astype(np.int32)
    bp, be = find_boundary_2d(tris)
    mask = np.zeros(len(x), dtype=bool)
    mask[:len(lo)] = lo[:, 1] <= 1e-12
    if segment:
        k = len(x)
        x = np.concatenate([x, [[-side, -gap], [2 * side, -gap]]])
        bp = np.concatenate([bp, [k, k + 1]]).astype(np.int32)
        be = np.concatenate([be, [[k, k + 1]]]).astype(np.int32)
        mask = np.concatenate([mask, [True, True]])
    v = np.zeros_like(x)
    v[len(lo):len(lo) + len(up), 1] = -speed
    x_rest = x.copy()
    return Scene2D('two_squares_2d', x, tris, v, bp, be, lambda t: (mask, x_rest), E=E, nu=nu, steps=steps,
                   meta={'seed': seed, 'n': n, 'angle': float(ang)})


def square_stack_2d(k=8, n=16, seed=0, side=0.1, gap=2e-3, jitter=0.1, steps=50):
    """A column of k squares (n x n quads, seed-drawn rotations up to 30 degrees and +-jitter
    horizontal offsets) stacked with ``gap`` between bounding circles above a fixed ground
    segment: the 2D workload for timing."""
    rng = np.random.default_rng(seed)
    base, bt = tri_grid(n, n, (side, side))
    r = np.sqrt(2) * side / 2
    xs, ts, y = [], [], gap + r
    for _ in range(k):
        R = _rot2(rng.uniform(-np.pi / 6, np.pi / 6))
        ctr = np.array([rng.uniform(-jitter, jitter) * side, y])
        ts.append(bt + sum(len(a) for a in xs))
        xs.append((base - side / 2) @ R.T + ctr)
        y += 2 * r + gap
    x = np.concatenate(xs)
    tris = np.concatenate(ts).astype(np.int32)
    bp, be = find_boundary_2d(tris)
    m = len(x)
    x = np.concatenate([x, [[-1.0, 0.0], [1.0, 0.0]]])
    bp = np.concatenate([bp, [m, m + 1]]).astype(np.int32)
    be = np.concatenate([be, [[m, m + 1]]]).astype(np.int32)
    mask = np.zeros(len(x), dtype=bool)
    mask[m:] = True
    x_rest = x.copy()
    return Scene2D('square_stack_2d', x, tris, np.zeros_like(x), bp, be, lambda t: (mask, x_rest), steps=steps,
                   meta={'seed': seed, 'k': k, 'n': n})
