"""Minimal Taichi-semantics shim that lets the reference's own Python kernels run on the CPU.

Test infrastructure only: it exists so that ``tests/golden/make_golden.py`` can execute the
reference solver's unmodified ``@ti.kernel`` / ``@ti.func`` source (loaded through
``oracle/ref_shim/loader.py``) and record golden vectors.  Nothing in the product imports it.

Semantics restated from Taichi 1.5.0 (``requirements.txt:10`` of the reference), the pieces the
particle-flow-map step uses:

* every field and every kernel scalar argument annotated ``float`` is f32; kernel arithmetic on
  f32 values with Python literals stays f32 (numpy's NEP 50 weak-scalar rule gives the same
  result as Taichi's constant folding into the default ``f32``);
* ``int()`` truncates toward zero (elementwise on vectors);
* the outermost ``for`` of a kernel is Taichi's parallel struct-for; here it runs sequentially in
  index order, which is one legal schedule, so float ``atomic_add`` / ``+=`` accumulate in that
  order;
* ``ti.Vector.unit`` is an integer vector; small-matrix products and dots are sequential sums
  without fused multiply-add.

Only what the reference's live step, its MGPCG class and its initial conditions touch is here.
"""
import itertools
import math as _math

import numpy as np

f32 = np.float32
i32 = np.int32
f64 = np.float64
u8 = np.uint8
cuda = "cuda"
cpu = "cpu"
gpu = "gpu"
ij = "ij"
ijk = "ijk"

_FLOAT_TOKENS = (float, f32, f64, "f32")
_INT_TOKENS = (int, i32, "i32")


def init(*args, **kwargs):
    return None


def _np_dtype(dtype):
    if dtype in _INT_TOKENS or dtype is int or getattr(dtype, "__name__", "") == "_ti_int":
        return np.int32
    return np.float32


class _Scope:
    depth = 0  # > 0 while a @ti.kernel body runs


_SCOPE = _Scope()


# ----------------------------------------------------------------------------------------------
# scalar helpers
# ----------------------------------------------------------------------------------------------
def _as_f32_if_float(x):
    if isinstance(x, float) or isinstance(x, np.float64):
        return np.float32(x)
    return x


def _ti_int(x):
    """Taichi ``int()``: truncation toward zero, elementwise on vectors."""
    if isinstance(x, _Value):
        return x._wrap(np.trunc(x.a).astype(np.int32))
    if isinstance(x, (np.floating, float)):
        return int(x)
    return int(x)


def cast(x, dtype):
    if isinstance(x, _Value):
        return x._wrap(x.a.astype(_np_dtype(dtype)))
    return _np_dtype(dtype)(x)


def _unary(fn):
    def op(x):
        if isinstance(x, _Value):
            return x._wrap(fn(x.a))
        return fn(_as_f32_if_float(x))
    return op


abs = _unary(np.abs)  # noqa: A001  (Taichi name)
sqrt = _unary(np.sqrt)
exp = _unary(np.exp)
cos = _unary(np.cos)
sin = _unary(np.sin)
floor = _unary(np.floor)
log = _unary(np.log)


def _binary(fn):
    def op(a, b):
        if isinstance(a, _Value) or isinstance(b, _Value):
            aa = a.a if isinstance(a, _Value) else a
            bb = b.a if isinstance(b, _Value) else b
            tmpl = a if isinstance(a, _Value) else b
            return tmpl._wrap(fn(aa, bb))
        return fn(a, b)
    return op


min = _binary(np.minimum)  # noqa: A001
max = _binary(np.maximum)  # noqa: A001


class _Math:
    pi = _math.pi

    @staticmethod
    def clamp(x, lo, hi):
        return max(min(x, hi), lo)


math = _Math()


def static(x, *args):
    return x


def random(dtype=float):
    raise RuntimeError("ti.random is not reproducible; the golden runs do not use it")


# ----------------------------------------------------------------------------------------------
# Vector / Matrix values
# ----------------------------------------------------------------------------------------------
def _norm_dtype(arr):
    if arr.dtype.kind == "f" and arr.dtype != np.float32:
        return arr.astype(np.float32)
    if arr.dtype.kind in "iub" and arr.dtype != np.int32:
        return arr.astype(np.int32)
    return arr


def _seq_dot(a, b):
    acc = a[0] * b[0]
    for t in range(1, a.shape[0]):
        acc = acc + a[t] * b[t]
    return acc


class _Value:
    """Small Taichi vector (1-D) or matrix (2-D) value backed by a numpy array."""

    __array_priority__ = 1000

    def __init__(self, data, dt=None):
        if isinstance(data, _Value):
            arr = data.a.copy()
        elif isinstance(data, np.ndarray):
            arr = data
        else:
            rows = [list(r.a) if isinstance(r, _Value) else r for r in data]
            is_float = any(isinstance(v, (float, np.floating)) for v in np.ravel(np.array(rows, dtype=object)))
            arr = np.array(rows, dtype=np.float32 if is_float else np.int32)
        if dt is not None:
            arr = arr.astype(_np_dtype(dt))
        self.a = _norm_dtype(np.asarray(arr))

    # construction ------------------------------------------------------------------------------
    def _wrap(self, arr):
        out = _Value.__new__(_Value)
        out.a = _norm_dtype(np.asarray(arr))
        return out

    @staticmethod
    def rows(vs):
        return _Value(np.stack([v.a for v in vs], axis=0))

    @staticmethod
    def cols(vs):
        return _Value(np.stack([v.a for v in vs], axis=1))

    @staticmethod
    def zero(dt, n, m=None):
        shape = (n,) if m is None else (n, m)
        return _Value(np.zeros(shape, dtype=_np_dtype(dt)))

    @staticmethod
    def unit(n, i, dt=None):
        arr = np.zeros(n, dtype=_np_dtype(dt) if dt is not None else np.int32)
        arr[i] = 1
        return _Value(arr)

    # element access ----------------------------------------------------------------------------
    def __getitem__(self, idx):
        r = self.a[idx]
        if isinstance(r, np.ndarray):
            return self._wrap(r)
        if isinstance(r, np.integer):
            return int(r)  # Taichi integer components combine with f32 as f32
        return r

    def __setitem__(self, idx, v):
        self.a[idx] = v.a if isinstance(v, _Value) else v

    def __getattr__(self, name):
        comp = {"x": 0, "y": 1, "z": 2, "w": 3}
        if name in comp:
            return self[comp[name]]
        if name in ("xyz", "xy"):
            return self._wrap(self.a[: len(name)])
        raise AttributeError(name)

    def __setattr__(self, name, v):
        comp = {"x": 0, "y": 1, "z": 2, "w": 3}
        if name in comp:
            self.a[comp[name]] = v
        elif name in ("xyz", "xy"):
            self.a[: len(name)] = v.a if isinstance(v, _Value) else v
        else:
            object.__setattr__(self, name, v)

    def __iter__(self):
        return iter(self.a)

    def __len__(self):
        return self.a.shape[0]

    @property
    def n(self):
        return self.a.shape[0]

    # arithmetic ---------------------------------------------------------------------------------
    def _bin(self, other, fn):
        o = other.a if isinstance(other, _Value) else other
        return self._wrap(fn(self.a, o))

    def _rbin(self, other, fn):
        o = other.a if isinstance(other, _Value) else other
        return self._wrap(fn(o, self.a))

    def __add__(self, o): return self._bin(o, np.add)
    def __radd__(self, o): return self._rbin(o, np.add)
    def __sub__(self, o): return self._bin(o, np.subtract)
    def __rsub__(self, o): return self._rbin(o, np.subtract)
    def __mul__(self, o): return self._bin(o, np.multiply)
    def __rmul__(self, o): return self._rbin(o, np.multiply)

    def __truediv__(self, o):
        r = self._bin(o, np.true_divide)
        return r

    def __rtruediv__(self, o): return self._rbin(o, np.true_divide)
    def __floordiv__(self, o): return self._bin(o, np.floor_divide)
    def __neg__(self): return self._wrap(-self.a)
    def __pow__(self, o): return self._bin(o, np.power)

    def __matmul__(self, other):
        A = self.a
        B = other.a
        if A.ndim == 2 and B.ndim == 1:
            return self._wrap(np.array([_seq_dot(A[r], B) for r in range(A.shape[0])], dtype=A.dtype))
        if A.ndim == 2 and B.ndim == 2:
            out = np.empty((A.shape[0], B.shape[1]), dtype=np.result_type(A, B))
            for r in range(A.shape[0]):
                for c in range(B.shape[1]):
                    out[r, c] = _seq_dot(A[r], B[:, c])
            return self._wrap(out)
        if A.ndim == 1 and B.ndim == 2:  # vector @ matrix: the vector as a row, v^T M
            return self._wrap(np.array([_seq_dot(A, B[:, c]) for c in range(B.shape[1])],
                                       dtype=np.result_type(A, B)))
        raise TypeError("unsupported matmul")

    # reductions / linear algebra ---------------------------------------------------------------
    def dot(self, other):
        return _seq_dot(self.a, other.a)

    def sum(self):
        acc = self.a.flat[0]
        for v in self.a.flat[1:]:
            acc = acc + v
        return int(acc) if isinstance(acc, np.integer) else acc

    def norm(self):
        return np.sqrt(self.dot(self))

    def normalized(self):
        return self / self.norm()

    def cross(self, o):
        a, b = self.a, o.a
        return self._wrap(np.array([a[1] * b[2] - a[2] * b[1],
                                    a[2] * b[0] - a[0] * b[2],
                                    a[0] * b[1] - a[1] * b[0]], dtype=np.result_type(a, b)))

    def outer_product(self, o):
        return self._wrap(np.outer(self.a, o.a))

    def transpose(self):
        return self._wrap(self.a.T.copy())

    def __repr__(self):
        return f"ti.Matrix({self.a!r})"


class Vector:
    """``ti.Vector`` namespace: constructs 1-D values and vector fields."""

    def __new__(cls, data, dt=None):
        return _Value(data, dt)

    @staticmethod
    def field(n, dtype=float, shape=None, **kw):
        return Field(dtype, shape, (n,))

    @staticmethod
    def unit(n, i, dt=None):
        return _Value.unit(n, i, dt)

    @staticmethod
    def zero(dt, n):
        return _Value.zero(dt, n)


class Matrix:
    """``ti.Matrix`` namespace: constructs 2-D values and matrix fields."""

    def __new__(cls, data, dt=None):
        return _Value(data, dt)

    rows = staticmethod(_Value.rows)
    cols = staticmethod(_Value.cols)
    zero = staticmethod(_Value.zero)
    unit = staticmethod(_Value.unit)

    @staticmethod
    def field(n, m, dtype=float, shape=None, **kw):
        return Field(dtype, shape, (n, m))


# ----------------------------------------------------------------------------------------------
# fields
# ----------------------------------------------------------------------------------------------
def _index(idx):
    if idx is None:
        return ()
    if isinstance(idx, _Value):
        return tuple(int(v) for v in idx.a)
    if isinstance(idx, tuple):
        out = []
        for v in idx:
            if isinstance(v, _Value):
                out.extend(int(x) for x in v.a)
            else:
                out.append(int(v))
        return tuple(out)
    return (int(idx),)


class Field:
    def __init__(self, dtype, shape, elem=()):
        self.dtype = _np_dtype(dtype)
        self.elem = tuple(elem)
        self.data = None
        if shape is not None:
            self._alloc(shape)

    def _alloc(self, shape):
        if isinstance(shape, int):
            shape = (shape,)
        self.shape = tuple(int(s) for s in shape)
        self.data = np.zeros(self.shape + self.elem, dtype=self.dtype)

    # Taichi API ----------------------------------------------------------------------------------
    def __getitem__(self, idx):
        r = self.data[_index(idx)]
        if self.elem:
            return _Value(r)  # a view: component writes go through, as in Taichi
        if _SCOPE.depth == 0:
            return r.item()  # Python-scope reads give Python float/int, as in Taichi
        return r

    def __setitem__(self, idx, v):
        self.data[_index(idx)] = v.a if isinstance(v, _Value) else v

    def __iter__(self):
        ranges = [range(s) for s in self.shape]
        if len(ranges) == 1:
            return iter(ranges[0])
        return itertools.product(*ranges)

    def fill(self, v):
        self.data[...] = v

    def to_numpy(self):
        return self.data.copy()

    def from_numpy(self, arr):
        self.data[...] = np.asarray(arr).astype(self.dtype)

    def copy_from(self, other):
        self.data[...] = other.data

    def to_torch(self, device=None):
        import torch
        return torch.from_numpy(self.data.copy())

    def from_torch(self, t):
        self.data[...] = t.detach().cpu().numpy().astype(self.dtype)


def field(dtype=float, shape=None, **kw):
    return Field(dtype, shape)


class _SNode:
    def __init__(self, shape=()):
        self.shape = tuple(shape)

    def pointer(self, indices, shape):
        if isinstance(shape, int):
            shape = (shape,)
        return _SNode(self.shape + tuple(shape) if self.shape else tuple(shape))

    def dense(self, indices, shape):
        if isinstance(shape, int):
            shape = (shape,) * (len(indices) if isinstance(indices, str) else 1)
        if not self.shape:
            return _SNode(tuple(shape))
        return _SNode(tuple(a * b for a, b in zip(self.shape, shape)))

    bitmasked = dense

    def place(self, *fields):
        for f in fields:
            f._alloc(self.shape)
        return self


root = _SNode()


def grouped(x):
    if isinstance(x, Field):
        ranges = [range(s) for s in x.shape]
    elif isinstance(x, _NdRange):
        ranges = x.ranges
    else:
        raise TypeError("grouped expects a field or ndrange")
    for t in itertools.product(*ranges):
        yield _Value(np.array(t, dtype=np.int32))


class _NdRange:
    def __init__(self, *args):
        self.ranges = []
        for a in args:
            if isinstance(a, (tuple, list)):
                self.ranges.append(range(int(a[0]), int(a[1])))
            else:
                self.ranges.append(range(int(a)))

    def __iter__(self):
        if len(self.ranges) == 1:
            return iter(self.ranges[0])
        return itertools.product(*self.ranges)


def ndrange(*args):
    return _NdRange(*args)


# atomics: the loader rewrites ``ti.atomic_op(F[idx], v)`` into ``_ti_atomic(op, F, idx, v)``
def _ti_atomic(op, target, idx, value):
    if isinstance(target, Field):
        old = target[idx]
        old_c = old.a.copy() if isinstance(old, _Value) else old
        if op == "add":
            target[idx] = old + value
        elif op == "max":
            target[idx] = max(old, value)
        elif op == "min":
            target[idx] = min(old, value)
        return old_c
    raise TypeError("atomic on a non-field target")


# ----------------------------------------------------------------------------------------------
# decorators and type tokens
# ----------------------------------------------------------------------------------------------
class _Template:
    pass


def template():
    return _Template()


class _Types:
    @staticmethod
    def vector(n, dtype=float):
        return ("vector", n, dtype)

    @staticmethod
    def matrix(n, m, dtype=float):
        return ("matrix", n, m, dtype)

    @staticmethod
    def ndarray(*a, **k):
        return ("ndarray",)


types = _Types()


def _coerce_arg(ann, v):
    if ann is float or ann is f32:
        return np.float32(v)
    if ann is int or ann is i32:
        return int(v)
    if isinstance(ann, tuple) and ann and ann[0] in ("vector", "matrix"):
        return _Value(np.array(v.a if isinstance(v, _Value) else v, dtype=np.float32))
    return v


def kernel(fn):
    import inspect
    sig = inspect.signature(fn)
    anns = {k: p.annotation for k, p in sig.parameters.items()}

    def wrapper(*args, **kwargs):
        bound = sig.bind(*args, **kwargs)
        for k in list(bound.arguments):
            bound.arguments[k] = _coerce_arg(anns.get(k), bound.arguments[k])
        _SCOPE.depth += 1
        try:
            return fn(*bound.args, **bound.kwargs)
        finally:
            _SCOPE.depth -= 1

    wrapper.__name__ = fn.__name__
    wrapper.__wrapped__ = fn
    return wrapper


def func(fn):
    return fn


def data_oriented(cls):
    return cls
