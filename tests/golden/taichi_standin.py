"""Numpy stand-in for the subset of the (pre-1.0) Taichi API that FastIPC's Newton path uses.

TEST INFRASTRUCTURE ONLY.  ``gen_golden.py`` uses this module to execute the reference's
own Python source (``common/math/distance.py``, ``ipc.py``, ``math_tools.py``,
``common/physics/neo_hookean.py``, ``projects/FastIPC/NEWTON_IPC.py``) in a container where
Taichi is not installed, so that golden vectors come from the reference's code rather than
from a restatement.  Nothing in the product imports it.

What it provides:
  * ``Mat`` – a numpy ``ndarray`` subclass with Taichi's small-matrix methods
    (``norm_sqr``, ``cross``, ``outer_product``, ``inverse`` ...).  Vectors are 1-D.
  * fields (``ti.field`` / ``ti.Vector.field`` / ``ti.Matrix.field``) backed by numpy arrays,
    laid out by ``ti.root.dense(...).place(...)``; the sparse spatial-hash grid of
    NEWTON_IPC.py (pointer/pointer/dense/dynamic SNodes) becomes a dict of python lists.
  * an import hook that loads reference modules with three source rewrites Taichi's
    AST transformer would otherwise perform:
      - ``ti.atomic_add(F[None], k)``       -> increments field F, returns the old value;
      - ``ti.atomic_min(a, e)`` (statement) -> ``a = min(a, e)``;
      - ``ti.external_func_call(func=f, args=A, outputs=(o1, ..))`` -> ``o1, .. = call(f, A)``
        through ctypes, with one ``double*`` per output (the reference ``a.so`` ABI);
    and module-level ``int``/``min``/``max``/``print`` that act elementwise on vectors
    (Taichi overloads these inside kernels).
  * ``ti.svd`` as a rotation-variant SVD (det U = det V = +1, sign folded into the last sigma) built
    on numpy; Taichi's own svd is third-party and absent.

Kernels run sequentially in Python; ``@ti.kernel`` parallel loops become plain loops.
"""
import ast
import builtins
import ctypes
import importlib.abc
import importlib.util
import itertools
import math
import sys

import numpy as np

np.seterr(all='ignore')

f64 = 'f64'
f32 = 'f32'
i32 = 'i32'
cpu = 'cpu'
gpu = 'gpu'
i = 'i'
ij = 'ij'
ijk = 'ijk'


def indices(*a):
    return a


def init(*a, **k):
    pass


def func(f):
    return f


def kernel(f):
    return f


def static(x, *rest):
    return x


def template():
    return None


class _Runtime:
    default_fp = f64


def get_runtime():
    return _Runtime()


class Mat(np.ndarray):
    """Taichi small matrix/vector value (1-D array = column vector)."""

    def __new__(cls, data):
        # taichi matrices are values: always copy so in-place edits never alias the input
        return np.array(data, dtype=np.float64).view(cls)

    @property
    def n(self):
        return self.shape[0]

    @property
    def m(self):
        return 1 if self.ndim == 1 else self.shape[1]

    def norm_sqr(self):
        return np.float64(np.sum(np.asarray(self) ** 2))

    def norm(self):
        return np.sqrt(self.norm_sqr())

    def dot(self, o):
        return np.float64(np.dot(np.asarray(self).ravel(), np.asarray(o).ravel()))

    def cross(self, o):
        a, b = np.asarray(self), np.asarray(o)
        if a.shape == (2,):   # taichi's 2D cross product is the scalar a0 b1 - a1 b0
            return np.float64(a[0] * b[1] - a[1] * b[0])
        return Mat(np.cross(a, b))

    def outer_product(self, o):
        return Mat(np.outer(np.asarray(self), np.asarray(o)))

    def inverse(self):
        # explicit adjugate / determinant like taichi's small-matrix inverse: a singular
        # matrix gives inf/nan entries instead of raising
        a = np.asarray(self)
        with np.errstate(divide='ignore', invalid='ignore'):
            if a.shape == (2, 2):
                inv_det = np.float64(1.0) / (a[0, 0] * a[1, 1] - a[0, 1] * a[1, 0])
                return Mat(inv_det * np.array([[a[1, 1], -a[0, 1]], [-a[1, 0], a[0, 0]]]))
            if a.shape == (3, 3):
                c = np.array([[a[1, 1] * a[2, 2] - a[1, 2] * a[2, 1], a[0, 2] * a[2, 1] - a[0, 1] * a[2, 2], a[0, 1] * a[1, 2] - a[0, 2] * a[1, 1]],
                              [a[1, 2] * a[2, 0] - a[1, 0] * a[2, 2], a[0, 0] * a[2, 2] - a[0, 2] * a[2, 0], a[0, 2] * a[1, 0] - a[0, 0] * a[1, 2]],
                              [a[1, 0] * a[2, 1] - a[1, 1] * a[2, 0], a[0, 1] * a[2, 0] - a[0, 0] * a[2, 1], a[0, 0] * a[1, 1] - a[0, 1] * a[1, 0]]])
                det = a[0, 0] * c[0, 0] + a[0, 1] * c[1, 0] + a[0, 2] * c[2, 0]
                return Mat(c * (np.float64(1.0) / det))
        return Mat(np.linalg.inv(a))

    def determinant(self):
        return np.float64(np.linalg.det(np.asarray(self)))

    def transpose(self):
        return Mat(np.asarray(self).T)

    def __getitem__(self, k):
        # a taichi vector is an n x 1 matrix: v[i, 0] is v[i]
        if self.ndim == 1 and isinstance(k, tuple) and len(k) == 2 and isinstance(k[1], (int, np.integer)) and k[1] == 0:
            k = k[0]
        r = np.ndarray.__getitem__(self, k)
        if isinstance(r, np.ndarray) and r.ndim == 0:
            return r[()]
        return r


class _BoolMat(np.ndarray):
    pass


class Matrix:
    def __new__(cls, data):
        a = np.asarray(data, dtype=np.float64)
        return Mat(a)

    @staticmethod
    def rows(rows):
        return Mat(np.stack([np.asarray(r, dtype=np.float64) for r in rows]))

    @staticmethod
    def zero(dtype, n, m=None):
        return Mat(np.zeros(n if m is None or m == 1 else (n, m)))

    @staticmethod
    def field(n, m, dtype):
        return Field(dtype, (n, m))


class Vector:
    def __new__(cls, data):
        a = np.array(data)
        if a.dtype.kind in 'iu':          # integer vectors (index tuples) stay integer
            return a.view(Mat)
        return Mat(a.astype(np.float64))

    @staticmethod
    def field(n, dtype):
        return Field(dtype, (n,))


def _wrap(r):
    if isinstance(r, np.ndarray):
        if r.ndim == 0:
            return r[()]
        return Mat(r) if r.dtype != bool else r
    return r


def min(*a):  # noqa: A001 - elementwise for vectors, like taichi
    if builtins.len(a) == 1:
        return builtins.min(a[0])
    if builtins.any(isinstance(v, np.ndarray) for v in a):
        r = np.asarray(a[0])
        for v in a[1:]:
            r = np.minimum(r, np.asarray(v))
        return _wrap(r)
    return builtins.min(*a)


def max(*a):  # noqa: A001
    if builtins.len(a) == 1:
        return builtins.max(a[0])
    if builtins.any(isinstance(v, np.ndarray) for v in a):
        r = np.asarray(a[0])
        for v in a[1:]:
            r = np.maximum(r, np.asarray(v))
        return _wrap(r)
    return builtins.max(*a)


def ti_int(v, *rest):
    if isinstance(v, np.ndarray):
        return np.asarray(v).astype(np.int64).view(np.ndarray)
    return builtins.int(v, *rest)


def sqrt(x):
    return _wrap(np.sqrt(x))


def log(x):
    return _wrap(np.log(x))


def pow(x, y):  # noqa: A001
    return _wrap(np.power(x, y))


def abs(x):  # noqa: A001
    return _wrap(np.abs(x))


def floor(x):
    return _wrap(np.floor(x))


def cast(x, dtype):
    return float(x) if dtype == f64 else builtins.int(x)


def svd(F):
    U, s, Vt = np.linalg.svd(np.asarray(F))
    V = Vt.T
    k = len(s) - 1          # the sign goes into the last singular value (2x2 and 3x3)
    if np.linalg.det(U) < 0:
        U[:, k] *= -1
        s[k] *= -1
    if np.linalg.det(V) < 0:
        V[:, k] *= -1
        s[k] *= -1
    return Mat(U), Mat(np.diag(s)), Mat(V)


def ndrange(*ranges):
    rs = [range(builtins.int(r[0]), builtins.int(r[1])) if isinstance(r, tuple) else range(builtins.int(r)) for r in ranges]
    return itertools.product(*rs)


def grouped(it):
    for t in it:
        yield np.array(t, dtype=np.int64)


# --------------------------------------------------------------------------- fields
class _Component:
    def __init__(self, f, d):
        self.f, self.d = f, d

    def __getitem__(self, k):
        return self.f.data[k, self.d]

    def __setitem__(self, k, v):
        self.f.data[k, self.d] = v


class Field:
    def __init__(self, dtype, elem=(), shape=None):
        self.dtype = dtype
        self.elem = tuple(elem)
        self.data = None
        if shape is not None:
            self._alloc(shape if isinstance(shape, tuple) else (shape,))

    def _alloc(self, shape):
        dt = np.int32 if self.dtype == i32 else np.float64
        self.data = np.zeros(tuple(shape) + self.elem, dtype=dt)

    @property
    def shape(self):
        return self.data.shape[:self.data.ndim - builtins.len(self.elem)]

    def __iter__(self):
        return iter(range(self.shape[0]))

    def __getitem__(self, k):
        if k is None:
            k = ()
        r = self.data[k]
        if self.elem:
            return Mat(r.copy())
        return r[()] if isinstance(r, np.ndarray) and r.ndim == 0 else r

    def __setitem__(self, k, v):
        if k is None:
            k = ()
        self.data[k] = np.asarray(v)

    def __call__(self, d):
        return _Component(self, d)

    def fill(self, v):
        self.data[...] = v

    def to_numpy(self):
        return self.data.copy()

    def from_numpy(self, a):
        a = np.asarray(a)
        if self.data is None or self.data.shape != a.shape:
            self.data = np.zeros(a.shape, dtype=self.data.dtype if self.data is not None else a.dtype)
        self.data[...] = a

    def parent(self):
        return self


def field(dtype, shape=None):
    return Field(dtype, (), shape)


class _DynamicCells:
    """The pointer/pointer/dense/dynamic sparse grid: cell index tuple -> list of ids."""

    def __init__(self):
        self.cells = {}
        self.off = (0, 0, 0)

    def deactivate_all(self):
        self.cells.clear()


class _SNode:
    def __init__(self, grid=None):
        self.grid = grid

    def dense(self, axes, n):
        return _SNode(self.grid) if self.grid is not None else _DenseSNode(n)

    def pointer(self, axes, n):
        g = self.grid if self.grid is not None else _DynamicCells()
        return _SNode(g)

    def dynamic(self, axes, n, chunk_size=None):
        return _SNode(self.grid)

    def place(self, *fields, offset=None):
        for f in fields:
            f.cells = self.grid
            f.off = tuple(offset[:-1]) if offset is not None else (0, 0, 0)
            f.__class__ = _PidField
        return self

    def deactivate_all(self):
        self.grid.deactivate_all()


class _DenseSNode:
    def __init__(self, n):
        self.n = n if isinstance(n, tuple) else (n,)

    def place(self, *fields, offset=None):
        for f in fields:
            f._alloc(self.n)
        return self


class _Root(_SNode):
    def dense(self, axes, n):
        return _DenseSNode(n)


root = _Root()


class _PidField(Field):
    def __getitem__(self, k):
        cell = tuple(builtins.int(k[d]) - self.off[d] for d in range(builtins.len(k) - 1))
        return self.cells.cells[cell][k[-1]]


def append(parent, I, v):
    parent.cells.cells.setdefault(tuple(builtins.int(t) for t in I), []).append(builtins.int(v))


def length(parent, I):
    return builtins.len(parent.cells.cells.get(tuple(builtins.int(t) for t in I), ()))


def atomic_add_field(f, k, v):
    old = f[k]
    f[k] = old + v
    return old


class GUI:
    def __init__(self, *a, **k):
        raise RuntimeError('GUI is not available (no graphics stack)')


# --------------------------------------------------------------------------- source rewrites
class _Rewriter(ast.NodeTransformer):
    def _is_ti(self, node, name):
        return (isinstance(node, ast.Attribute) and node.attr == name
                and isinstance(node.value, ast.Name) and node.value.id == 'ti')

    def visit_Call(self, node):
        self.generic_visit(node)
        if self._is_ti(node.func, 'atomic_add') and isinstance(node.args[0], ast.Subscript):
            sub = node.args[0]
            key = sub.slice
            return ast.copy_location(ast.Call(
                func=ast.Attribute(value=ast.Name(id='ti', ctx=ast.Load()), attr='atomic_add_field', ctx=ast.Load()),
                args=[sub.value, key, node.args[1]], keywords=[]), node)
        return node

    def visit_Expr(self, node):
        self.generic_visit(node)
        call = node.value
        if isinstance(call, ast.Call) and self._is_ti(call.func, 'atomic_min'):
            target = call.args[0]
            return ast.copy_location(ast.Assign(
                targets=[ast.Name(id=target.id, ctx=ast.Store())],
                value=ast.Call(func=ast.Name(id='min', ctx=ast.Load()), args=[ast.Name(id=target.id, ctx=ast.Load()), call.args[1]], keywords=[])), node)
        if isinstance(call, ast.Call) and self._is_ti(call.func, 'external_func_call'):
            kw = {k.arg: k.value for k in call.keywords}
            outs = kw['outputs'].elts
            tgt = ast.Tuple(elts=[ast.Name(id=o.id, ctx=ast.Store()) for o in outs], ctx=ast.Store())
            val = ast.Call(func=ast.Attribute(value=ast.Name(id='ti', ctx=ast.Load()), attr='ext_call', ctx=ast.Load()),
                           args=[kw['func'], kw['args'], ast.Constant(builtins.len(outs))], keywords=[])
            return ast.copy_location(ast.Assign(targets=[tgt], value=val), node)
        return node


def ext_call(fn, args, n_out):
    outs = [ctypes.c_double(0.0) for _ in range(n_out)]
    cargs = [ctypes.c_double(float(a)) for a in args] + [ctypes.byref(o) for o in outs]
    fn.restype = None
    fn(*cargs)
    return tuple(o.value for o in outs)


_quiet_print = lambda *a, **k: None  # noqa: E731


class ReferenceLoader(importlib.abc.Loader):
    """Loads a reference module with the rewrites above and elementwise builtins."""

    def __init__(self, path, substitutions=(), quiet=True):
        self.path = path
        self.subs = substitutions
        self.quiet = quiet

    def create_module(self, spec):
        return None

    def exec_module(self, module):
        src = open(self.path).read()
        for a, b in self.subs:
            if a not in src:
                raise RuntimeError(f'substitution target not found in {self.path}: {a!r}')
            src = src.replace(a, b)
        tree = _Rewriter().visit(ast.parse(src, filename=self.path))
        ast.fix_missing_locations(tree)
        module.__dict__.update({'int': ti_int, 'min': min, 'max': max})
        if self.quiet:
            module.__dict__['print'] = _quiet_print
        exec(compile(tree, self.path, 'exec'), module.__dict__)


class ReferenceFinder(importlib.abc.MetaPathFinder):
    def __init__(self, mapping):
        self.mapping = mapping  # module name -> (path, substitutions)

    def find_spec(self, name, path=None, target=None):
        if name in self.mapping:
            p, subs = self.mapping[name]
            return importlib.util.spec_from_file_location(name, p, loader=ReferenceLoader(p, subs))
        return None


def install(mapping):
    """Register this module as ``taichi`` and route the given reference modules through
    the rewriting loader.  ``mapping``: module name -> (source path, [(old, new), ...])."""
    sys.modules['taichi'] = sys.modules[__name__]
    finder = ReferenceFinder(mapping)
    sys.meta_path.insert(0, finder)
    return finder
