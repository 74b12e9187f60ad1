"""Adaptive, diagonally equilibrated FSAI: P = G^T G (warp_preconditioners/fsai.py).

Setup is one libgbpc call per stage: adaptive factor rows (warp per row, fused
row sort), CSR packing, optional factor compression with validation, and the
explicit transpose.  Apply is the fused G -> G^T product.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib
from .linear import LinearOperator
from .sparse import BsrMatrix, bsr_transposed, scalarize

_PIVOT_FLOOR = {torch.float32: 1.0e-6, torch.float64: 1.0e-12}


def fsai_rows(scalar: BsrMatrix, width: int, step: int, kap: float, pivot_floor: float):
    """Adaptive factor rows: returns (ell_cols, ell_vals, row_counts, scale, status[3])."""
    n = scalar.nrow
    dev = scalar.device
    dt = scalar.scalar_type
    cols = torch.empty(n * width, dtype=torch.int32, device=dev)
    vals = torch.empty(n * width, dtype=dt, device=dev)
    counts = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    scale = torch.empty(max(n, 1), dtype=dt, device=dev)
    status = (ctypes.c_int32 * 3)()
    rc = _lib.load().gbpc_fsai_setup(
        n, _lib.ptr(scalar.offsets), _lib.ptr(scalar.columns), _lib.ptr(scalar.values),
        _lib.dtype_code(dt), width, step, float(kap), float(pivot_floor), _lib.ptr(cols),
        _lib.ptr(vals), _lib.ptr(counts), _lib.ptr(scale), status, _lib.stream(dev))
    return cols, vals, counts, scale, list(status), rc


def pack_rows(n, width, cols, vals, counts) -> BsrMatrix:
    """Sorted ELL rows -> canonical CSR (fsai_pack.py:58-71)."""
    dev = vals.device
    off = torch.empty(n + 1, dtype=torch.int32, device=dev)
    nnz = ctypes.c_int64()
    code = _lib.dtype_code(vals.dtype)
    _lib.call("gbpc_fsai_pack", n, width, _lib.ptr(cols), _lib.ptr(vals), _lib.ptr(counts), code,
              _lib.ptr(off), None, None, ctypes.byref(nnz), _lib.stream(dev))
    col = torch.empty(nnz.value, dtype=torch.int32, device=dev)
    val = torch.empty(nnz.value, dtype=vals.dtype, device=dev)
    _lib.call("gbpc_fsai_pack", n, width, _lib.ptr(cols), _lib.ptr(vals), _lib.ptr(counts), code,
              _lib.ptr(off), _lib.ptr(col), _lib.ptr(val), ctypes.byref(nnz), _lib.stream(dev))
    return BsrMatrix(n, n, (1, 1), off, col, val)


def convert_factor(g: BsrMatrix, dtype: torch.dtype) -> BsrMatrix:
    """Narrow the factor storage and validate it (fsai.py:181-196, :343-355)."""
    out = torch.empty(g.nnz, dtype=dtype, device=g.device)
    bad = ctypes.c_int32()
    _lib.call("gbpc_convert_factor", g.nrow, _lib.ptr(g.offsets), _lib.ptr(g.columns),
              _lib.ptr(g.values), _lib.dtype_code(g.scalar_type), _lib.ptr(out),
              _lib.dtype_code(dtype), ctypes.byref(bad), _lib.stream(g.device), what="FSAI")
    return BsrMatrix(g.nrow, g.ncol, (1, 1), g.offsets, g.columns, out)


class FSAI(LinearOperator):
    """Approximate inverse ``G.T @ G`` of an SPD BSR matrix.

    Same constructor as warp_preconditioners.FSAI (fsai.py:241-251):
    ``max_row_size`` includes the diagonal; each search selects up to
    ``max_step_size`` distinct largest-residual entries from the lower
    triangular frontier; ``kap_tolerance`` tests the relative energy
    improvement after each batch (zero disables it); square blocks are
    scalarised keeping stored zeros.  float32 and float64 matrices are
    supported.  ``factor_dtype`` may be the matrix type, float32 for a float64
    matrix (products still accumulate in float64), or bfloat16 (an addition of
    this build for the mixed-precision path).  ``apply_lanes`` is validated for
    compatibility; the apply kernel's layout is chosen by the library.
    Setup synchronises; apply is stream-ordered and graph-capturable.
    """

    def __init__(self, A, max_row_size=8, kap_tolerance=1.0e-3, pivot_floor=None, apply_lanes=1,
                 factor_dtype=None, reuse_pattern=False, max_step_size=1):
        if (not isinstance(A, BsrMatrix) or A.shape[0] != A.shape[1]
                or A.block_shape[0] != A.block_shape[1]):
            raise ValueError("FSAI requires a square BSR matrix with square blocks")
        if A.scalar_type not in (torch.float32, torch.float64):
            raise TypeError("FSAI supports float32 and float64")
        if isinstance(max_row_size, bool) or not isinstance(max_row_size, int) \
                or not 1 <= max_row_size <= 64:
            raise ValueError("max_row_size must be an integer in [1, 64]")
        if isinstance(max_step_size, bool) or not isinstance(max_step_size, int) \
                or not 1 <= max_step_size <= 64:
            raise ValueError("max_step_size must be an integer in [1, 64]")
        if not 0 <= kap_tolerance < 1:
            raise ValueError("kap_tolerance must be in [0, 1)")
        if pivot_floor is None:
            pivot_floor = _PIVOT_FLOOR[A.scalar_type]
        if not 0 < pivot_floor < 1:
            raise ValueError("pivot_floor must be in (0, 1)")
        if not isinstance(apply_lanes, int) or apply_lanes not in (1, 2, 4, 8, 16, 32):
            raise ValueError("apply_lanes must be one of 1, 2, 4, 8, 16, 32")
        if factor_dtype is None:
            factor_dtype = A.scalar_type
        if factor_dtype != A.scalar_type and not (
            A.scalar_type == torch.float64 and factor_dtype in (torch.float32, torch.bfloat16)
        ):
            raise ValueError(
                "factor_dtype must be the matrix scalar type, or torch.float32 for a float64 matrix"
            )
        if reuse_pattern:
            raise NotImplementedError("reuse_pattern (fixed-support refit) is not available yet")
        self.max_row_size = max_row_size
        self.max_step_size = max_step_size
        self.factor_dtype = factor_dtype
        self.apply_lanes = apply_lanes
        self.source = A
        scalar = scalarize(A)
        n = scalar.nrow
        dt = scalar.scalar_type
        cols, vals, counts, scale, status, rc = fsai_rows(scalar, max_row_size, max_step_size,
                                                          kap_tolerance, pivot_floor)
        if rc == _lib.ERR_DIAGONAL or status[0]:
            raise ValueError(f"FSAI requires finite positive diagonals ({status[0]} invalid rows)")
        if rc == _lib.ERR_FACTOR or status[2]:
            raise ValueError("FSAI factor lost finite entries or a positive diagonal")
        _lib.check(rc, "FSAI")
        self.truncated_rows = int(status[1])
        self.scale = scale[:n]
        self.G = pack_rows(n, max_row_size, cols, vals, counts)
        if factor_dtype != dt:
            self.G = convert_factor(self.G, factor_dtype)
        self.GT = bsr_transposed(self.G)
        self._op = _lib.new_op(
            "gbpc_op_fsai", n, 1, _lib.ptr(self.G.offsets), _lib.ptr(self.G.columns),
            _lib.ptr(self.G.values), _lib.ptr(self.GT.offsets), _lib.ptr(self.GT.columns),
            _lib.ptr(self.GT.values), _lib.dtype_code(factor_dtype), _lib.dtype_code(dt),
            _lib.stream(A.device))
        super().__init__(A.shape, dt, A.device, self._apply)

    def _apply(self, x, y, z, alpha, beta):
        self._op.apply(x.reshape(-1), y.reshape(-1) if y is not None else None, z.view(-1),
                       alpha, beta, self.device)
