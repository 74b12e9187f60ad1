"""ctypes binding of libgbpc.so (declared in include/gbpc.h).

The library is the only compute path: importing an operator without a loadable
libgbpc.so, or calling it without a CUDA device, raises instead of falling back
to any host implementation.
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

import torch

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libgbpc.so"

GBPC_F64, GBPC_F32, GBPC_BF16 = 0, 1, 2
GBPC_F32_APPLY = 3  # float64 vectors, float32 arithmetic inside (preconditioners)
GBPC_CG, GBPC_CR = 0, 1

OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_DIAGONAL = 3
ERR_FACTOR = 4
ERR_CONVERSION = 5
ERR_PIVOT = 6
ERR_FREE_INDEX = 7
ERR_MASS = 8
ERR_TIMEOUT = 9
ERR_NOMEM = 10
ERR_UNSUPPORTED = 11
ERR_BLOCK_PIVOT = 12

_VALUE_ERRORS = {
    ERR_ARG, ERR_DIAGONAL, ERR_FACTOR, ERR_CONVERSION, ERR_PIVOT, ERR_FREE_INDEX, ERR_MASS,
    ERR_BLOCK_PIVOT, ERR_UNSUPPORTED,
}

_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p
_int = ctypes.c_int
_dbl = ctypes.c_double
_szp = ctypes.POINTER(ctypes.c_size_t)

# name -> argtypes (all functions return int status)
_SIGNATURES = {
    "gbpc_version": [],
    "gbpc_device_bytes": [_szp],
    "gbpc_fsai_setup": [_int, _vp, _vp, _vp, _int, _int, _int, _dbl, _dbl, _vp, _vp, _vp, _vp,
                        _i32p, _vp],
    "gbpc_fsai_pack": [_int, _int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _i64p, _vp],
    "gbpc_csr_transpose": [_int, _int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _vp],
    "gbpc_scalarize": [_int, _int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _vp],
    "gbpc_convert_factor": [_int, _vp, _vp, _vp, _int, _vp, _int, _i32p, _vp],
    "gbpc_fsai_refit": [_int, _vp, _vp, _vp, _int, _vp, _vp, _int, _dbl, _vp, _int, _i32p, _vp],
    "gbpc_transpose_map": [_int, _vp, _vp, _vp, _vp, _vp, _vp],
    "gbpc_spgemm": [_int, _int, _vp, _vp, _vp, _vp, _int, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                    _i64p, _vp],
    "gbpc_scatter_values": [ctypes.c_int64, _vp, _vp, _vp, _int, _vp],
    "gbpc_op_fsai_refill": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _int, _vp],
    "gbpc_op_sparse": [_int, _int, _int, _vp, _vp, _vp, _int, _int, _vp, ctypes.POINTER(_vp)],
    "gbpc_op_fsai": [_int, _int, _vp, _vp, _vp, _vp, _vp, _vp, _int, _int, _vp,
                     ctypes.POINTER(_vp)],
    "gbpc_op_sqlap": [_int, _vp, _vp, _vp, _int, _vp, _vp, _int, _dbl, _vp, ctypes.POINTER(_vp)],
    "gbpc_sqlap_rhs": [_vp, _vp, _vp, _vp],
    "gbpc_op_diagonal": [_int, _int, _vp, _vp, _vp, _int, _vp, ctypes.POINTER(_vp)],
    "gbpc_op_block_jacobi": [_int, _int, _vp, _vp, _vp, _int, _dbl, _vp, _vp, ctypes.POINTER(_vp)],
    "gbpc_op_block_jacobi_update": [_vp, _int, _int, _vp, _vp, _vp, _int, _dbl, _vp, _vp],
    "gbpc_op_matching_schur": [_int, _int, _vp, _vp, _vp, _int, _vp, _vp, _vp,
                               ctypes.POINTER(_vp)],
    "gbpc_op_shifted_block": [_int, _int, _dbl, _int, _vp, _vp, ctypes.POINTER(_vp)],
    "gbpc_op_bilu0": [_int, _int, _vp, _vp, _vp, _int, _int, _int, _dbl, _dbl, _vp, _vp, _vp,
                      ctypes.POINTER(_vp)],
    "gbpc_block_fsai_setup": [_int, _int, _int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _vp, _vp],
    "gbpc_csr_to_bsr": [_int, _int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _i64p, _vp],
    "gbpc_bsr_transpose": [_int, _int, _int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _vp],
    "gbpc_op_apply": [_vp, _vp, _vp, _vp, _dbl, _dbl, _vp],
    "gbpc_op_rows": [_vp, _i64p],
    "gbpc_op_device_bytes": [_vp, _szp],
    "gbpc_op_destroy": [_vp],
    "gbpc_krylov": [_int, _vp, _vp, _vp, _vp, _dbl, _dbl, _int, _int, _vp, _vp, _vp, _i32p, _dp,
                    _dp, _vp],
    "gbpc_solver_create": [_int, _vp, _vp, _int, _int, _vp, ctypes.POINTER(_vp)],
    "gbpc_solver_run": [_vp, _vp, _vp, _dbl, _dbl, _int, _vp, _vp, _vp, _vp],
    "gbpc_solver_destroy": [_vp],
    "gbpc_solver_set_history": [_vp, _vp, _int],
    "gbpc_solver_cluster": [_vp, ctypes.POINTER(_int)],
    "gbpc_solver_device_bytes": [_vp, _szp],
    "gbpc_gmres_create": [_vp, _vp, _int, _vp, ctypes.POINTER(_vp)],
    "gbpc_gmres_run": [_vp, _vp, _vp, _dbl, _dbl, _int, _int, _vp, _vp, _vp, _vp],
    "gbpc_gmres_device_bytes": [_vp, _szp],
    "gbpc_gmres_destroy": [_vp],
    "gbpc_bop_sparse": [_int, _vp, _vp, _vp, _int, _int, _int, _vp, ctypes.POINTER(_vp)],
    "gbpc_bop_fsai": [_int, _vp, _vp, _vp, _vp, _vp, _vp, _int, _int, _int, _int, _vp,
                      ctypes.POINTER(_vp)],
    "gbpc_bop_sqlap": [_int, _vp, _vp, _vp, _int, _int, _int, _vp, _dbl, _int, _vp,
                       ctypes.POINTER(_vp)],
    "gbpc_bop_apply": [_vp, _int, _vp, _vp, _vp, _dbl, _dbl, _vp],
    "gbpc_bop_device_bytes": [_vp, _szp],
    "gbpc_bop_destroy": [_vp],
    "gbpc_bsolver_create": [_vp, _vp, _int, _int, _vp, ctypes.POINTER(_vp)],
    "gbpc_bsolver_run": [_vp, _int, _vp, _vp, _dbl, _dbl, _int, _vp, _vp, _vp],
    "gbpc_bsolver_device_bytes": [_vp, _szp],
    "gbpc_bsolver_destroy": [_vp],
    "gbpc_refine": [_vp, _vp, _int, _vp, _vp, _dbl, _dbl, _int, _int, _i32p, _i32p, _vp],
    "gbpc_rademacher": [ctypes.c_int64, _int, _int, _vp, _vp],
    "gbpc_vec_axpby": [ctypes.c_int64, _int, _dbl, _vp, _dbl, _vp, _vp, _vp],
    "gbpc_vec_dot_work_size": [],
    "gbpc_vec_dot": [ctypes.c_int64, _int, _vp, _vp, _vp, _vp, _vp],
    "gbpc_fma_probe": [ctypes.c_int64, _int, _vp, _vp],
    "gbpc_msolver_create": [_vp, _vp, _int, _i64p, _int, _int, _vp, ctypes.POINTER(_vp)],
    "gbpc_msolver_run": [_vp, _vp, _vp, _dbl, _dbl, _int, _vp, _vp, _vp, _vp],
    "gbpc_msolver_device_bytes": [_vp, _szp],
    "gbpc_msolver_destroy": [_vp],
    "gbpc_csolver_create": [_int, _vp, _vp, _vp, ctypes.POINTER(_vp)],
    "gbpc_csolver_run": [_vp, _int, _vp, _vp, _dbl, _dbl, _int, _vp, _vp, _vp, _vp],
    "gbpc_csolver_cluster_size": [_vp, ctypes.POINTER(_int)],
    "gbpc_csolver_device_bytes": [_vp, _szp],
    "gbpc_csolver_destroy": [_vp],
}

_lock = threading.Lock()
_lib = None


class GbpcError(RuntimeError):
    """A CUDA-level failure inside libgbpc."""


def load():
    """Load libgbpc.so, building it first when the sources are newer."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        from . import _build

        path = _build.build()
        lib = ctypes.CDLL(str(path))
        lib.gbpc_last_error.restype = ctypes.c_char_p
        lib.gbpc_last_error.argtypes = []
        for name, args in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _lib = lib
        return lib


def last_error() -> str:
    return load().gbpc_last_error().decode()


def check(rc: int, what: str = "") -> None:
    """Raise the reference's exception type for a non-zero status."""
    if rc == OK:
        return
    msg = last_error()
    if what:
        msg = f"{what}: {msg}"
    if rc in _VALUE_ERRORS:
        raise ValueError(msg)
    if rc == ERR_NOMEM:
        raise MemoryError(msg)
    raise GbpcError(msg)


def call(name: str, *args, what: str | None = None) -> None:
    check(getattr(load(), name)(*args), what or name)


def dtype_code(dtype: torch.dtype) -> int:
    if dtype == torch.float64:
        return GBPC_F64
    if dtype == torch.float32:
        return GBPC_F32
    if dtype == torch.bfloat16:
        return GBPC_BF16
    raise TypeError(f"unsupported dtype {dtype}")


def ptr(t: torch.Tensor | None):
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("libgbpc operates on CUDA tensors; got a tensor on " + str(t.device))
    if not t.is_contiguous():
        raise ValueError("libgbpc needs contiguous tensors")
    return ctypes.c_void_p(t.data_ptr())


def stream(device=None):
    """The current torch stream of `device`, as the C ABI's void*."""
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def object_bytes(getter: str, handle) -> int:
    """Device bytes held by a library object (`getter` is its *_device_bytes)."""
    out = ctypes.c_size_t()
    call(getter, handle, ctypes.byref(out))
    return int(out.value)


def live_device_bytes() -> int:
    """Device bytes held by every live allocation of the library."""
    out = ctypes.c_size_t()
    call("gbpc_device_bytes", ctypes.byref(out))
    return int(out.value)


class OpHandle:
    """Owns a gbpc_op*."""

    def __init__(self, handle: ctypes.c_void_p, rows: int):
        self.handle = handle
        self.rows = rows

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _lib is not None:
            try:
                _lib.gbpc_op_destroy(h)
            except Exception:
                pass
            self.handle = None

    @property
    def device_bytes(self) -> int:
        return object_bytes("gbpc_op_device_bytes", self.handle)

    def apply(self, x, y, z, alpha, beta, device=None):
        check(load().gbpc_op_apply(self.handle, ptr(x), ptr(y) if y is not None else None, ptr(z),
                                   float(alpha), float(beta), stream(device)), "apply")


def new_op(name: str, *args, what: str | None = None) -> OpHandle:
    out = ctypes.c_void_p()
    call(name, *args, ctypes.byref(out), what=what)
    rows = ctypes.c_int64()
    check(load().gbpc_op_rows(out, ctypes.byref(rows)))
    return OpHandle(out, rows.value)
