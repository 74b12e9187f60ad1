"""Scalar, vector and matrix types of the Warp emulation (test infrastructure).

Scalars are NumPy scalar types (one IEEE rounding per operation, in the
scalar's precision).  ``vector(length, dtype)`` and ``matrix(shape, dtype)``
return value classes; their products sum in increasing index order
(``(A x)_i = A_i0 x_0 + A_i1 x_1 + ...``), each product and sum rounded on
its own.  Determinants and inverses of 2x2..4x4 blocks use cofactor
expansion (the adjugate over the determinant).
"""

from __future__ import annotations

from functools import lru_cache

import numpy as np

float16 = np.float16
float32 = np.float32
float64 = np.float64
int32 = np.int32
int64 = np.int64
uint32 = np.uint32
bool_ = np.bool_
int8 = np.int8
uint8 = np.uint8


def normalize_dtype(dtype):
    if dtype is int:
        return int32
    if dtype is float:
        return float32
    if dtype is bool:
        return bool_
    return dtype


def scalar_of(dtype):
    dtype = normalize_dtype(dtype)
    if isinstance(dtype, type) and issubclass(dtype, (Vec, Mat)):
        return dtype._dtype
    return dtype


def type_shape(dtype):
    dtype = normalize_dtype(dtype)
    if isinstance(dtype, type) and issubclass(dtype, (Vec, Mat)):
        return dtype._shape
    return ()


def type_length(dtype):
    shape = type_shape(dtype)
    return int(np.prod(shape)) if shape else 1


def type_scalar_type(dtype):
    return scalar_of(dtype)


def type_size_in_bytes(dtype):
    return type_length(dtype) * np.dtype(scalar_of(dtype)).itemsize


def types_equal(a, b, match_generic=False):
    return normalize_dtype(a) is normalize_dtype(b)


def _coerce(cls, args):
    if len(args) == 0:
        return np.zeros(cls._shape, dtype=cls._dtype)
    if len(args) == 1:
        x = args[0]
        if isinstance(x, Mat):
            return np.array(x.a, dtype=cls._dtype).reshape(cls._shape)
        if isinstance(x, np.ndarray) or isinstance(x, (list, tuple)):
            return np.array(x, dtype=cls._dtype).reshape(cls._shape)
        return np.full(cls._shape, x, dtype=cls._dtype)
    comps = []
    for x in args:
        if isinstance(x, Mat):
            comps.extend(x.a.ravel().tolist())
        elif isinstance(x, Vec):
            comps.extend(list(x))
        else:
            comps.append(x)
    return np.array(comps, dtype=cls._dtype).reshape(cls._shape)


def _scalar_like(x):
    return not isinstance(x, (Vec, Mat))


class Vec(list):
    """A Warp vector value: a list of typed scalars (C-speed element access)."""

    _shape = (0,)
    _dtype = float64
    __array_ufunc__ = None  # NumPy scalars defer to the reflected operators

    def __init__(self, *args):
        t = self._dtype
        n = self._shape[0]
        if len(args) == 0:
            super().__init__([t(0)] * n)
        elif len(args) == 1:
            x = args[0]
            if isinstance(x, (Vec, list, tuple, np.ndarray)):
                vals = np.asarray(x, dtype=t).reshape(n)
                super().__init__(vals.tolist() if self._isint else list(vals))
            else:
                v = int(x) if self._isint else t(x)
                super().__init__([v] * n)
        else:
            vals = np.asarray(args, dtype=t).reshape(n)
            super().__init__(vals.tolist() if self._isint else list(vals))

    _isint = False

    @property
    def a(self):
        return np.array(self, dtype=self._dtype)

    def _new(self, arr):
        return type(self)(arr)

    def __add__(self, o):
        return self._new(self.a + o.a)

    def __iadd__(self, o):
        return self.__add__(o)

    def __sub__(self, o):
        return self._new(self.a - o.a)

    def __isub__(self, o):
        return self.__sub__(o)

    def __neg__(self):
        return self._new(-self.a)

    def __mul__(self, o):
        if _scalar_like(o):
            return self._new(self.a * self._dtype(o))
        if isinstance(o, Mat):  # row vector times matrix
            return _vec_mat(self, o)
        raise TypeError("vector * vector is not defined (use cw_mul)")

    def __imul__(self, o):
        return self.__mul__(o)

    def __rmul__(self, o):
        if _scalar_like(o):
            return self._new(self._dtype(o) * self.a)
        raise TypeError

    def __truediv__(self, o):
        with np.errstate(all="ignore"):
            return self._new(self.a / self._dtype(o))

    def __eq__(self, o):
        return isinstance(o, Vec) and bool(np.array_equal(self.a, o.a))

    __hash__ = None

    def __repr__(self):
        return f"vec{self._shape[0]}({list(self)})"


class Mat:
    _shape = (0, 0)
    _dtype = float64
    __slots__ = ("a",)
    __array_ufunc__ = None

    def __init__(self, *args):
        self.a = _coerce(type(self), args)

    def __getitem__(self, idx):
        if isinstance(idx, tuple):
            return self.a[idx]
        return vector(self._shape[1], self._dtype)(self.a[idx])

    def __setitem__(self, idx, v):
        if isinstance(v, Vec):
            v = v.a
        self.a[idx] = v

    def _new(self, arr, cls=None):
        cls = cls or type(self)
        out = object.__new__(cls)
        out.a = arr.astype(self._dtype, copy=False)
        return out

    def __add__(self, o):
        return self._new(self.a + o.a)

    def __sub__(self, o):
        return self._new(self.a - o.a)

    def __neg__(self):
        return self._new(-self.a)

    def __mul__(self, o):
        if _scalar_like(o):
            return self._new(self.a * self._dtype(o))
        if isinstance(o, Vec):
            return _mat_vec(self, o)
        return _mat_mat(self, o)

    def __rmul__(self, o):
        if _scalar_like(o):
            return self._new(self._dtype(o) * self.a)
        raise TypeError

    def __matmul__(self, o):
        return self.__mul__(o)

    def __truediv__(self, o):
        with np.errstate(all="ignore"):
            return self._new(self.a / self._dtype(o))

    def __eq__(self, o):
        return isinstance(o, Mat) and bool(np.array_equal(self.a, o.a))

    def __repr__(self):
        return f"mat{self._shape}({self.a.tolist()})"


def _mat_vec(m, v):
    a, x = m.a, v.a
    with np.errstate(all="ignore"):
        acc = a[:, 0] * x[0]
        for j in range(1, a.shape[1]):
            acc = acc + a[:, j] * x[j]
    return vector(a.shape[0], m._dtype)(acc)


def _vec_mat(v, m):
    a, x = m.a, v.a
    with np.errstate(all="ignore"):
        acc = x[0] * a[0, :]
        for j in range(1, a.shape[0]):
            acc = acc + x[j] * a[j, :]
    return vector(a.shape[1], m._dtype)(acc)


def _mat_mat(m, o):
    a, b = m.a, o.a
    with np.errstate(all="ignore"):
        acc = a[:, 0:1] * b[0:1, :]
        for k in range(1, a.shape[1]):
            acc = acc + a[:, k:k + 1] * b[k:k + 1, :]
    return matrix((a.shape[0], b.shape[1]), m._dtype)(acc)


@lru_cache(None)
def vector(length, dtype=float32):
    dtype = normalize_dtype(dtype)
    isint = np.dtype(dtype).kind in "iub"
    return type(f"vec{length}_{np.dtype(dtype).name}", (Vec,),
                {"_shape": (int(length),), "_dtype": dtype, "_isint": isint})


@lru_cache(None)
def matrix(shape, dtype=float32):
    dtype = normalize_dtype(dtype)
    shape = tuple(int(s) for s in shape)
    return type(f"mat{shape[0]}{shape[1]}_{np.dtype(dtype).name}", (Mat,),
                {"_shape": shape, "_dtype": dtype, "__slots__": ()})


vec2 = vector(2, float32)
vec3 = vector(3, float32)
vec2d = vector(2, float64)
vec3d = vector(3, float64)
vec4d = vector(4, float64)
vec2i = vector(2, int32)
vec3i = vector(3, int32)
vec4i = vector(4, int32)
mat22 = matrix((2, 2), float32)
mat33 = matrix((3, 3), float32)
mat22d = matrix((2, 2), float64)
mat33d = matrix((3, 3), float64)
mat44d = matrix((4, 4), float64)


def dot(a, b):
    x, y = a.a, b.a
    acc = x[0] * y[0]
    for i in range(1, len(x)):
        acc = acc + x[i] * y[i]
    return acc


def cross(a, b):
    x, y = a.a, b.a
    return type(a)(x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0])


def transpose(m):
    return matrix((m._shape[1], m._shape[0]), m._dtype)(m.a.T.copy())


def outer(a, b):
    return matrix((a._shape[0], b._shape[0]), a._dtype)(np.outer(a.a, b.a))


def diag(v):
    return matrix((v._shape[0], v._shape[0]), v._dtype)(np.diag(v.a))


def _det(a):
    n = a.shape[0]
    if n == 1:
        return a[0, 0]
    if n == 2:
        return a[0, 0] * a[1, 1] - a[0, 1] * a[1, 0]
    total = None
    for c in range(n):
        minor = np.delete(np.delete(a, 0, axis=0), c, axis=1)
        term = a[0, c] * _det(minor)
        if total is None:
            total = term
        elif c % 2:
            total = total - term
        else:
            total = total + term
    return total


def determinant(m):
    with np.errstate(all="ignore"):
        return _det(m.a)


def inverse(m):
    a = m.a
    n = a.shape[0]
    with np.errstate(all="ignore"):
        det = _det(a)
        if det == 0:
            return type(m)()
        out = np.empty_like(a)
        for r in range(n):
            for c in range(n):
                minor = np.delete(np.delete(a, c, axis=0), r, axis=1)
                cof = _det(minor) if n > 1 else a.dtype.type(1)
                out[r, c] = (cof if (r + c) % 2 == 0 else -cof) / det
    return type(m)(out)
