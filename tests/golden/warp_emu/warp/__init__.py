"""A NumPy emulation of the parts of NVIDIA Warp that the reference library uses.

TEST INFRASTRUCTURE ONLY.  The reference (warp_preconditioners) is pure Python
whose kernels are ``@wp.kernel`` functions compiled by warp-lang (PyPI
``warp-lang>=1.15``, not installable here).  This package lets the reference's
own source run unmodified on the host: a kernel is executed by calling its
Python function once per thread index, in launch order, with ``wp.tid()``
returning that index.  Scalars follow the C types Warp compiles to:

* float64 values are NumPy float64 scalars and float32 values NumPy float32
  scalars, so every ``+ - * /`` and ``sqrt`` is one IEEE operation rounded to
  the scalar's type, evaluated in source order with no multiply-add
  contraction (what Warp's CPU backend computes);
* ints are Python ints (the reference's indices stay far below 2^31);
* vector and matrix locals (``wp.types.vector`` / ``wp.types.matrix``) are
  value types; reading an array element copies it.

Threads run one after another, so kernels that only write their own outputs
and use atomics for counters (every reference kernel on the CPU path) get
Warp's results.  Tile primitives are CUDA-only in the reference and are not
emulated.  Only the "cpu" device exists.

The semantics restated here (array views, BSR formats, the Krylov solvers in
``warp.optim.linear``) follow Warp's public documentation; no Warp source is
reproduced.  Used by tests/golden/make_reference_golden.py and
tests/golden/run_reference_tests.py, never by the product.
"""

from __future__ import annotations

import builtins
import math
from contextlib import contextmanager

import numpy as np

from . import types
from .types import (  # noqa: F401
    Mat,
    Vec,
    bool_,
    float16,
    float32,
    float64,
    int32,
    int64,
    mat22,
    mat22d,
    mat33,
    mat33d,
    mat44d,
    matrix,
    normalize_dtype,
    scalar_of,
    type_length,
    type_shape,
    uint32,
    vec2,
    vec2d,
    vec3,
    vec3d,
    vec4d,
    vec2i,
    vec3i,
    vec4i,
    vector,
)

__version__ = "emulated"

LOG_WARNING = 2
LOG_INFO = 1


class _Config:
    log_level = LOG_WARNING
    quiet = True
    mode = "release"
    verify_fp = False


config = _Config()


def init():
    return None


# ---------------------------------------------------------------- devices


class Device:
    def __init__(self, alias):
        self.alias = alias

    is_cuda = False
    is_cpu = True
    ordinal = -1

    def __eq__(self, other):
        if isinstance(other, Device):
            return self.alias == other.alias
        if isinstance(other, str):
            return other == self.alias
        return NotImplemented

    def __hash__(self):
        return hash(self.alias)

    def __repr__(self):
        return self.alias

    __str__ = __repr__


_CPU = Device("cpu")
_current = [_CPU]


def get_device(device=None):
    if device is None:
        return _current[-1]
    if isinstance(device, Device):
        return device
    if isinstance(device, str) and device == "cpu":
        return _CPU
    raise RuntimeError(f"emulated Warp has no device {device!r} (cpu only)")


def get_preferred_device():
    return _CPU


def is_cuda_available():
    return False


def is_cpu_available():
    return True


def get_cuda_device_count():
    return 0


def synchronize():
    return None


def synchronize_device(device=None):
    return None


class ScopedDevice:
    def __init__(self, device):
        self.device = get_device(device)

    def __enter__(self):
        _current.append(self.device)
        return self.device

    def __exit__(self, *exc):
        _current.pop()
        return False


class ScopedCapture:
    def __init__(self, *a, **k):
        raise RuntimeError("graph capture needs CUDA (not emulated)")


def capture_launch(graph, *a, **k):
    raise RuntimeError("graph capture needs CUDA (not emulated)")


class ScopedTimer:
    def __init__(self, *a, **k):
        self.elapsed = 0.0

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


def set_module_options(*a, **k):
    return None


# ---------------------------------------------------------------- arrays


class array:
    """A typed view of a NumPy buffer: ``shape`` counts elements, each element
    being a scalar, vector or matrix of ``dtype``.  Views (``view``,
    ``reshape``, ``flatten``, slices) share the buffer, so ``ptr`` identifies
    aliasing exactly as Warp's device pointers do."""

    def __init__(self, data=None, dtype=None, shape=None, device=None, ndim=None,
                 copy=True, _buffer=None, **kwargs):
        if dtype is None and data is not None and not isinstance(data, array):
            arr = np.asarray(data)
            dtype = {np.dtype(np.float64): float64, np.dtype(np.float32): float32,
                     np.dtype(np.int32): int32, np.dtype(np.int64): int32,
                     np.dtype(np.float16): float16, np.dtype(np.bool_): bool_}[arr.dtype]
        self.dtype = normalize_dtype(dtype) if dtype is not None else float32
        self.device = get_device(device)
        self._elem = type_shape(self.dtype)
        base = scalar_of(self.dtype)
        if _buffer is not None:
            self._np = _buffer
        elif data is None and shape is None:
            self._np = None  # a type annotation inside a kernel signature
            self._ndim = ndim or 1
            return
        elif data is None:
            if isinstance(shape, int):
                shape = (shape,)
            self._np = np.zeros(tuple(shape) + self._elem, dtype=base)
        else:
            if isinstance(data, array):
                data = data._np
            arr = np.array(data, dtype=base, copy=True)
            ne = len(self._elem)
            if ne and arr.ndim >= ne and arr.shape[arr.ndim - ne:] == self._elem:
                pass
            elif ne:
                arr = arr.reshape((-1,) + self._elem)
            self._np = arr
        self._ndim = self._np.ndim - len(self._elem)
        self._isint = np.issubdtype(self._np.dtype, np.integer) or self._np.dtype == np.bool_
        self._vtype = None
        if self._elem:
            self._vtype = self.dtype

    # -- metadata
    @property
    def shape(self):
        return self._np.shape[: self._ndim]

    @property
    def ndim(self):
        return self._ndim

    @property
    def size(self):
        return int(np.prod(self.shape)) if self._ndim else 1

    @property
    def ptr(self):
        return self._np.__array_interface__["data"][0] if self._np.size else 0

    @property
    def strides(self):
        return self._np.strides[: self._ndim]

    @property
    def is_contiguous(self):
        return self._np.flags["C_CONTIGUOUS"]

    def __len__(self):
        return self.shape[0]

    # -- element access (host and kernel)
    def __getitem__(self, idx):
        if type(idx) is int:  # the kernel fast path
            if self._isint:
                return self._np.item(idx)
            if self._vtype is None:
                return self._np[idx]
            return self._vtype(self._np[idx])
        if isinstance(idx, slice) or (isinstance(idx, tuple) and any(isinstance(i, slice)
                                                                     for i in idx)):
            return array(dtype=self.dtype, device=self.device, _buffer=self._np[idx])
        if not isinstance(idx, tuple):
            idx = int(idx)
        else:
            idx = tuple(int(i) for i in idx)
        if self._isint:
            return self._np.item(idx) if not isinstance(idx, tuple) else self._np.item(*idx)
        v = self._np[idx]
        if self._vtype is not None:
            return self._vtype(v)
        return v

    def __setitem__(self, idx, value):
        if self._vtype is not None and isinstance(value, Mat):
            self._np[idx] = value.a
        elif self._vtype is not None and isinstance(value, Vec):
            self._np[idx] = list(value)
        else:
            self._np[idx] = value

    # -- host API
    def numpy(self):
        return self._np

    def list(self):
        return self._np.tolist()

    def zero_(self):
        self._np[...] = 0

    def fill_(self, value):
        if isinstance(value, (Vec, Mat)):
            self._np[...] = value.a
        else:
            self._np[...] = value

    def assign(self, src):
        src = src._np if isinstance(src, array) else np.asarray(src)
        self._np[...] = src.reshape(self._np.shape)

    def view(self, dtype):
        dtype = normalize_dtype(dtype)
        new_elem = type_shape(dtype)
        count = int(np.prod(self._elem)) if self._elem else 1
        new_count = int(np.prod(new_elem)) if new_elem else 1
        shape = self.shape
        if self._ndim == 0:
            shape = (1,)
        last = shape[-1] * count // new_count
        buf = self._np.reshape(tuple(shape[:-1]) + (last,) + new_elem)
        return array(dtype=dtype, device=self.device, _buffer=buf)

    def flatten(self):
        return array(dtype=self.dtype, device=self.device,
                     _buffer=self._np.reshape((-1,) + self._elem))

    def reshape(self, shape):
        if isinstance(shape, int):
            shape = (shape,)
        return array(dtype=self.dtype, device=self.device,
                     _buffer=self._np.reshape(tuple(shape) + self._elem))

    def contiguous(self):
        return self

    def to(self, device):
        get_device(device)
        return self

    def __array__(self, dtype=None, copy=None):
        return np.asarray(self._np, dtype=dtype)

    def __repr__(self):
        return f"wp.array({self._np!r}, dtype={getattr(self.dtype, '__name__', self.dtype)})"


def array1d(*a, **k):
    return array(*a, ndim=1, **k)


def array2d(*a, **k):
    return array(*a, ndim=2, **k)


def empty(shape=0, dtype=float32, device=None, **k):
    return array(dtype=dtype, shape=shape, device=device)


def zeros(shape=0, dtype=float32, device=None, **k):
    return array(dtype=dtype, shape=shape, device=device)


def ones(shape=0, dtype=float32, device=None, **k):
    out = array(dtype=dtype, shape=shape, device=device)
    out._np[...] = 1
    return out


def full(shape=0, value=0, dtype=None, device=None, **k):
    if dtype is None:
        dtype = float32 if isinstance(value, float) else int32
    out = array(dtype=dtype, shape=shape, device=device)
    out.fill_(value)
    return out


def empty_like(a, device=None, **k):
    return array(dtype=a.dtype, shape=a.shape, device=device or a.device)


def zeros_like(a, device=None, **k):
    return array(dtype=a.dtype, shape=a.shape, device=device or a.device)


def ones_like(a, device=None, **k):
    return ones(a.shape, a.dtype, device or a.device)


def full_like(a, value, device=None, **k):
    return full(a.shape, value, a.dtype, device or a.device)


def clone(a, device=None, **k):
    return array(dtype=a.dtype, device=device or a.device, _buffer=a._np.copy())


def copy(dest, src, dest_offset=0, src_offset=0, count=0):
    d = dest._np.reshape((-1,) + dest._elem)
    s = src._np.reshape((-1,) + src._elem)
    if count == 0:
        count = s.shape[0] - src_offset
    d[dest_offset: dest_offset + count] = s[src_offset: src_offset + count]


def from_numpy(arr, dtype=None, shape=None, device=None, **k):
    return array(arr, dtype=dtype, device=device)


# ---------------------------------------------------------------- kernels

_tid = [0]


def tid():
    return _tid[0]


class Kernel:
    def __init__(self, func, **options):
        self.func = func
        self.key = func.__name__
        self.options = options

    def __call__(self, *args):
        return self.func(*args)


def kernel(f=None, *, enable_backward=None, module=None, **options):
    if f is None:
        return lambda g: Kernel(g)
    return Kernel(f)


def func(f=None, **options):
    if f is None:
        return lambda g: g
    return f


def overload(*a, **k):
    raise NotImplementedError("wp.overload is not emulated")


def struct(cls):
    return cls


def constant(x):
    return x


def static(x):
    return x


def _kernel_view(a):
    """What a kernel sees of an argument.  Scalar arrays are handed over as
    their buffers (a memoryview for integers, whose elements read as Python
    ints; the NumPy array itself for floats, whose elements read as typed
    NumPy scalars), so element access runs at C speed; vector and matrix
    arrays stay wrapped so that their elements read as value types."""
    if isinstance(a, array) and a._vtype is None and a._np is not None:
        if a._isint and a._np.size:
            return memoryview(a._np)
        return a._np
    return a


def launch(kernel, dim=None, inputs=(), outputs=(), device=None, block_dim=None, stream=None,
           record_tape=True, max_blocks=0, **k):
    get_device(device)
    fn = kernel.func if isinstance(kernel, Kernel) else kernel
    args = [_kernel_view(a) for a in list(inputs) + list(outputs)]
    if isinstance(dim, (tuple, list)):
        dims = tuple(int(d) for d in dim)
    else:
        dims = (int(dim),)
    if len(dims) == 1:
        for i in range(dims[0]):
            _tid[0] = i
            fn(*args)
    else:
        for idx in np.ndindex(*dims):
            _tid[0] = tuple(int(i) for i in idx)
            fn(*args)


def launch_tiled(*a, **k):
    raise NotImplementedError("tile launches need CUDA (not emulated)")


# ---------------------------------------------------------------- builtins


def _np_scalar(x):
    return x


def abs(x):  # noqa: A001
    if isinstance(x, (Vec, Mat)):
        return type(x)(np.abs(x.a))
    return builtins.abs(x)


def sqrt(x):
    if isinstance(x, (np.floating,)):
        with np.errstate(all="ignore"):
            return np.sqrt(x)
    with np.errstate(all="ignore"):
        return np.sqrt(np.float32(x)) if isinstance(x, int) else np.sqrt(x)


def min(a, b=None):  # noqa: A001
    if b is None:
        return a.a.min()
    return a if a < b else b


def max(a, b=None):  # noqa: A001
    if b is None:
        return a.a.max()
    return a if a > b else b


def clamp(x, lo, hi):
    return lo if x < lo else hi if x > hi else x


def isfinite(x):
    if isinstance(x, (Vec, Mat)):
        return bool(np.isfinite(x.a).all())
    return bool(np.isfinite(x))


def isnan(x):
    if isinstance(x, (Vec, Mat)):
        return bool(np.isnan(x.a).any())
    return bool(np.isnan(x))


def isinf(x):
    return bool(np.isinf(x))


def floor(x):
    return type(x)(np.floor(x))


def exp(x):
    return np.exp(x)


def log(x):
    return np.log(x)


def sin(x):
    return np.sin(x)


def cos(x):
    return np.cos(x)


def sign(x):
    return type(x)(np.sign(x))


def atomic_add(arr, *idx_and_value):
    *idx, value = idx_and_value
    idx = tuple(idx) if len(idx) > 1 else idx[0]
    old = arr[idx]
    arr[idx] = old + value
    return old


def atomic_sub(arr, *idx_and_value):
    *idx, value = idx_and_value
    idx = tuple(idx) if len(idx) > 1 else idx[0]
    old = arr[idx]
    arr[idx] = old - value
    return old


def atomic_max(arr, *idx_and_value):
    *idx, value = idx_and_value
    idx = tuple(idx) if len(idx) > 1 else idx[0]
    old = arr[idx]
    if value > old:
        arr[idx] = value
    return old


def atomic_min(arr, *idx_and_value):
    *idx, value = idx_and_value
    idx = tuple(idx) if len(idx) > 1 else idx[0]
    old = arr[idx]
    if value < old:
        arr[idx] = value
    return old


def atomic_cas(arr, *args):
    *idx, compare, value = args
    idx = tuple(idx) if len(idx) > 1 else idx[0]
    old = arr[idx]
    if old == compare:
        arr[idx] = value
    return old


def dot(a, b):
    return types.dot(a, b)


def cross(a, b):
    return types.cross(a, b)


def length(a):
    return sqrt(types.dot(a, a))


def transpose(m):
    return types.transpose(m)


def determinant(m):
    return types.determinant(m)


def inverse(m):
    return types.inverse(m)


def cw_mul(a, b):
    return type(a)(a.a * b.a)


def cw_div(a, b):
    return type(a)(a.a / b.a)


def outer(a, b):
    return types.outer(a, b)


def diag(v):
    return types.diag(v)


def identity(n, dtype):
    return matrix(shape=(n, n), dtype=dtype)(np.eye(n))


def select(cond, a, b):
    return b if cond else a


def where(cond, a, b):
    return a if cond else b


# ---------------------------------------------------------------- random numbers
#
# The PCG hash of Jarzynski and Olano ("Hash Functions for GPU Rendering",
# JCGT 2020), which Warp's documented rand_init / randi streams are built on:
# a state is seeded from (seed, offset) and each draw advances it by one hash.

_M32 = 0xFFFFFFFF


def _pcg(state):
    state = (state * 747796405 + 2891336453) & _M32
    word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & _M32
    return ((word >> 22) ^ word) & _M32


class _RandState:
    __slots__ = ("s",)

    def __init__(self, s):
        self.s = s & _M32


def rand_init(seed, offset=None):
    if offset is None:
        return _RandState(_pcg(seed & _M32))
    return _RandState(_pcg((seed + _pcg(offset & _M32)) & _M32))


def randi(state, lo=None, hi=None):
    state.s = _pcg(state.s)
    value = state.s - (1 << 32) if state.s >= (1 << 31) else state.s
    if lo is None:
        return value
    return lo + (state.s % (hi - lo))


# ---------------------------------------------------------------- submodules
from . import sparse, utils  # noqa: E402,F401
from . import optim  # noqa: E402,F401

math = math
