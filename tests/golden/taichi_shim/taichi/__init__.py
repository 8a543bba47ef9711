"""A minimal pure-Python stand-in for the ``taichi`` package (test infrastructure).

Taichi is not installed in this environment, so the Tichi_SPH reference modules
(``sph_config.py``, ``sph_util.py``, ``sph_obj.py``, ``sph.py``) cannot be imported
as shipped.  This shim implements just the subset of Taichi's Python surface those
modules use, and executes every ``@ti.kernel`` / ``@ti.func`` body as ordinary
sequential Python.  It exists only so ``tests/golden/make_golden.py`` can run the
reference's own kernel code and record golden vectors; nothing in the product
imports it.

Semantics it reproduces (the ones the reference's arithmetic depends on):

* fields are dense numpy arrays; ``float`` fields use ``TAICHI_SHIM_FP`` storage
  (``f64`` by default, ``f32`` to mimic Taichi's ``default_fp=f32`` stores);
* a Vector field element is a live view, so ``field[i][j] = v`` writes through;
* ``int(vector)`` truncates each component toward zero (Taichi's ``fptosi``);
* ``a // b`` on floats is ``floor(a / b)`` (Taichi's lowering, not Python's divmod rule);
* ``ti.atomic_add(f[idx], v)`` / ``atomic_min`` mutate the field element and
  return the old value -- the kernel source is rewritten through the ``ast``
  module (as Taichi itself does) so the subscript is passed by reference;
* the outermost ``for`` loops run serially, which equals Taichi's parallel loop
  up to the order of floating-point atomics (no reference kernel reads what a
  sibling iteration writes, except through atomics).
"""
import ast
import functools
import inspect
import math
import os
import textwrap

import numpy as np

_FP = np.float32 if os.environ.get("TAICHI_SHIM_FP", "f64") == "f32" else np.float64

# arch / dtype / axis tokens ---------------------------------------------------------
cpu = "cpu"
gpu = "gpu"
f32 = "f32"
f64 = "f64"
i32 = "i32"
i64 = "i64"
i = "axis_i"
j = "axis_j"
k = "axis_k"


def init(*args, **kwargs):
    return None


def _np_dtype(dt):
    if dt is float or dt in (f32, f64):
        return _FP
    if dt is int or dt in (i32, i64):
        return np.int32
    raise TypeError("taichi shim: unsupported dtype %r" % (dt,))


def _norm_shape(shape):
    if shape is None:
        return None
    if isinstance(shape, (int, np.integer)):
        return (int(shape),)
    return tuple(int(s) for s in shape)


def _key(k):
    if k is None:
        return ()
    if isinstance(k, tuple):
        return tuple(int(x) for x in k)
    return (int(k),)


def _py(v, dtype):
    return float(v) if np.issubdtype(dtype, np.floating) else int(v)


# Vector ------------------------------------------------------------------------------
class Vector:
    """Small value-semantics vector (a view when it came from a field element)."""

    __slots__ = ("a",)

    def __init__(self, values, dt=None):
        if isinstance(values, Vector):
            self.a = values.a.copy()
        else:
            arr = np.array(values)
            if arr.dtype == np.bool_:
                arr = arr.astype(np.int64)
            if np.issubdtype(arr.dtype, np.floating):
                arr = arr.astype(np.float64)
            elif np.issubdtype(arr.dtype, np.integer):
                arr = arr.astype(np.int64)
            self.a = arr

    @staticmethod
    def field(n, dtype, shape=None):
        return VectorField(n, dtype, shape)

    @classmethod
    def _wrap(cls, arr):
        v = cls.__new__(cls)
        v.a = arr
        return v

    @property
    def n(self):
        return self.a.shape[0]

    def __len__(self):
        return self.a.shape[0]

    def __getitem__(self, idx):
        v = self.a[int(idx)]
        return float(v) if np.issubdtype(self.a.dtype, np.floating) else int(v)

    def __setitem__(self, idx, v):
        self.a[int(idx)] = v

    def __iter__(self):
        return iter([self[x] for x in range(len(self))])

    @staticmethod
    def _o(x):
        return x.a if isinstance(x, Vector) else x

    def _promote(self):
        a = self.a
        if np.issubdtype(a.dtype, np.floating):
            return a.astype(np.float64)
        return a.astype(np.int64)

    def __add__(self, o):
        return Vector._wrap(self._promote() + Vector._o(o))

    __radd__ = __add__

    def __sub__(self, o):
        return Vector._wrap(self._promote() - Vector._o(o))

    def __rsub__(self, o):
        return Vector._wrap(Vector._o(o) - self._promote())

    def __mul__(self, o):
        return Vector._wrap(self._promote() * Vector._o(o))

    __rmul__ = __mul__

    def __truediv__(self, o):
        return Vector._wrap(self._promote() / Vector._o(o))

    def __rtruediv__(self, o):
        return Vector._wrap(Vector._o(o) / self._promote())

    def __floordiv__(self, o):
        a, b = self._promote(), Vector._o(o)
        if np.issubdtype(a.dtype, np.floating) or np.issubdtype(np.asarray(b).dtype, np.floating):
            # Taichi lowers float floordiv to floor(a / b), not Python's divmod rule
            return Vector._wrap(np.floor(a / b))
        return Vector._wrap(a // b)

    def __neg__(self):
        return Vector._wrap(-self._promote())

    def dot(self, o):
        r = np.dot(self._promote(), Vector._o(o))
        return float(r) if np.issubdtype(np.asarray(r).dtype, np.floating) else int(r)

    def norm_sqr(self):
        a = self._promote().astype(np.float64)
        return float(np.dot(a, a))

    def norm(self):
        return math.sqrt(self.norm_sqr())

    def normalized(self):
        a = self._promote().astype(np.float64)
        return Vector._wrap(a / math.sqrt(float(np.dot(a, a))))

    def to_numpy(self):
        return self.a.copy()

    def __repr__(self):
        return "Vector(%r)" % (self.a.tolist(),)


# fields --------------------------------------------------------------------------------
class _FieldBase:
    def _alloc(self, shape):
        self.shape = _norm_shape(shape)
        self.data = np.zeros(self.shape + self._tail, dtype=self.dtype)

    def fill(self, v):
        self.data[...] = v

    def to_numpy(self):
        return self.data.copy()

    def from_numpy(self, arr):
        self.data[...] = np.asarray(arr).reshape(self.data.shape)


class ScalarField(_FieldBase):
    _tail = ()

    def __init__(self, dtype, shape=None):
        self.dtype = _np_dtype(dtype)
        self.shape = None
        if shape is not None:
            self._alloc(shape)

    def __getitem__(self, k):
        return _py(self.data[_key(k)], self.dtype)

    def __setitem__(self, k, v):
        self.data[_key(k)] = v


class VectorField(_FieldBase):
    def __init__(self, n, dtype, shape=None):
        self.n = int(n)
        self._tail = (self.n,)
        self.dtype = _np_dtype(dtype)
        self.shape = None
        if shape is not None:
            self._alloc(shape)

    def __getitem__(self, k):
        return Vector._wrap(self.data[_key(k)])

    def __setitem__(self, k, v):
        self.data[_key(k)] = Vector._o(v) if isinstance(v, Vector) else np.asarray(v)


def field(dtype, shape=None):
    return ScalarField(dtype, shape)


class _Dense:
    def __init__(self, shape):
        self.shape = shape

    def dense(self, axis, n):
        return _Dense(self.shape + (int(n),))

    def place(self, *fields):
        for f in fields:
            f._alloc(self.shape)
        return self


class _Root:
    def dense(self, axis, n):
        return _Dense((int(n),))


root = _Root()


# helpers used by kernels ----------------------------------------------------------------
def static(x, *args):
    return x


def template():
    return None


def ext_arr():
    return None


def data_oriented(cls):
    return cls


def ceil(x):
    if isinstance(x, Vector):
        return Vector._wrap(np.ceil(x._promote().astype(np.float64)))
    return math.ceil(x)


def floor(x):
    if isinstance(x, Vector):
        return Vector._wrap(np.floor(x._promote().astype(np.float64)))
    return math.floor(x)


def sqrt(x):
    return math.sqrt(x)


def _shim_int(x):
    if isinstance(x, Vector):
        return Vector._wrap(np.trunc(x._promote()).astype(np.int64))
    return int(x)


def _shim_float(x):
    if isinstance(x, Vector):
        return Vector._wrap(x._promote().astype(np.float64))
    return float(x)


def _shim_atomic_add(container, idx, v):
    old = container[idx]
    container[idx] = old + v
    return old


def _shim_atomic_min(container, idx, v):
    old = container[idx]
    container[idx] = min(old, v)
    return old


def _shim_atomic_max(container, idx, v):
    old = container[idx]
    container[idx] = max(old, v)
    return old


def atomic_add(*a, **k):
    raise RuntimeError("taichi shim: atomic_add outside a transformed kernel")


def atomic_min(*a, **k):
    raise RuntimeError("taichi shim: atomic_min outside a transformed kernel")


def atomic_max(*a, **k):
    raise RuntimeError("taichi shim: atomic_max outside a transformed kernel")


_HELPERS = {
    "_shim_int": _shim_int,
    "_shim_float": _shim_float,
    "_shim_atomic_add": _shim_atomic_add,
    "_shim_atomic_min": _shim_atomic_min,
    "_shim_atomic_max": _shim_atomic_max,
}


def _call_name(func):
    if isinstance(func, ast.Name):
        return func.id
    if isinstance(func, ast.Attribute):
        return func.attr
    return None


class _Rewriter(ast.NodeTransformer):
    """Rewrites int()/float() casts and atomics on subscripts (pass-by-reference)."""

    def visit_Call(self, node):
        self.generic_visit(node)
        name = _call_name(node.func)
        if isinstance(node.func, ast.Name) and name in ("int", "float"):
            node.func = ast.Name(id="_shim_" + name, ctx=ast.Load())
            return node
        if name in ("atomic_add", "atomic_min", "atomic_max") and node.args:
            tgt = node.args[0]
            if isinstance(tgt, ast.Subscript):
                idx = tgt.slice
                return ast.copy_location(
                    ast.Call(func=ast.Name(id="_shim_" + name, ctx=ast.Load()),
                             args=[tgt.value, idx] + node.args[1:], keywords=[]),
                    node)
        return node


def _compile(fn):
    src = textwrap.dedent(inspect.getsource(fn))
    tree = ast.parse(src)
    fdef = tree.body[0]
    fdef.decorator_list = []
    for a in fdef.args.args + fdef.args.kwonlyargs:
        a.annotation = None
    fdef.returns = None
    tree = ast.fix_missing_locations(_Rewriter().visit(tree))
    g = fn.__globals__
    for k_, v_ in _HELPERS.items():
        g.setdefault(k_, v_)
    code = compile(tree, filename=inspect.getsourcefile(fn) or "<kernel>", mode="exec")
    ns = {}
    exec(code, g, ns)
    return ns[fdef.name]


class _Kernel:
    def __init__(self, fn):
        self.fn = fn
        self.compiled = None
        functools.update_wrapper(self, fn)

    def __get__(self, obj, objtype=None):
        if obj is None:
            return self
        return functools.partial(self.__call__, obj)

    def __call__(self, *args, **kwargs):
        if self.compiled is None:
            self.compiled = _compile(self.fn)
        return self.compiled(*args, **kwargs)


def kernel(fn):
    return _Kernel(fn)


def func(fn):
    return _Kernel(fn)


def grouped(f):
    return np.ndindex(*f.shape)
