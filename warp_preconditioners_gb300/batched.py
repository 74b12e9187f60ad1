"""Many right-hand sides of one system: batched operators, batched PCG and
mixed-precision iterative refinement.

Vectors are ``[n, k]`` row-major tensors with ``k <= 32``.  A group of
k-rounded-up-to-a-power-of-two lanes serves all k right-hand sides of a
matrix row, so matrix bytes are read once per iteration for the whole batch.  ``MixedPrecisionSolver`` runs the inner PCG in
float32 (float32 operator, float32 or bfloat16 FSAI factor, float64 dots) and
corrects in float64 with the float64 factored operator: iterative refinement
recovers float64 accuracy (componentwise backward error ~1e-15 on the
smoothing system) from float32 inner solves.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib
from .fsai import FSAI
from .sparse import BsrMatrix

MAX_RHS = 32


class BatchedOperator:
    """Z = alpha * Op X + beta * Y for [n, k] blocks of vectors."""

    def __init__(self, handle, rows, vector_dtype, device, max_rhs=MAX_RHS):
        self._h = handle
        self.rows = rows
        self.dtype = vector_dtype
        self.device = device
        self.max_rhs = max_rhs

    @property
    def device_bytes(self) -> int:
        return _lib.object_bytes("gbpc_bop_device_bytes", self._h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib._lib is not None:
            try:
                _lib._lib.gbpc_bop_destroy(h)
            except Exception:
                pass

    def apply(self, X, Y, Z, alpha=1.0, beta=0.0):
        k = _check_block(X, self.rows, self.dtype, self.max_rhs)
        _lib.call("gbpc_bop_apply", self._h, k, _lib.ptr(X), _lib.ptr(Y) if Y is not None else None,
                  _lib.ptr(Z), float(alpha), float(beta), _lib.stream(self.device))
        return Z


def _check_block(X, rows, dtype, max_rhs=MAX_RHS):
    if X.dim() != 2 or X.shape[0] != rows or not 1 <= X.shape[1] <= max_rhs:
        raise ValueError(f"expected an [{rows}, k] block with 1 <= k <= {max_rhs}")
    if X.dtype != dtype:
        raise TypeError(f"expected {dtype} vectors, got {X.dtype}")
    return int(X.shape[1])


def _new(name, *args, rows, vdt, device, max_rhs=MAX_RHS):
    out = ctypes.c_void_p()
    _lib.call(name, *args, ctypes.byref(out))
    return BatchedOperator(out, rows, vdt, device, max_rhs)


def _max_rhs(max_rhs):
    if isinstance(max_rhs, bool) or not isinstance(max_rhs, int) or not 1 <= max_rhs <= MAX_RHS:
        raise ValueError(f"max_rhs must be an integer in [1, {MAX_RHS}]")
    return max_rhs


def batched_sparse(A: BsrMatrix, value_dtype=None, vector_dtype=None) -> BatchedOperator:
    if A.block_shape != (1, 1):
        raise ValueError("batched operators take scalar CSR matrices")
    value_dtype = value_dtype or A.scalar_type
    vector_dtype = vector_dtype or (torch.float64 if value_dtype == torch.float64 else torch.float32)
    return _new("gbpc_bop_sparse", A.nrow, _lib.ptr(A.offsets), _lib.ptr(A.columns),
                _lib.ptr(A.values), _lib.dtype_code(A.scalar_type), _lib.dtype_code(value_dtype),
                _lib.dtype_code(vector_dtype), _lib.stream(A.device),
                rows=A.nrow, vdt=vector_dtype, device=A.device)


def batched_fsai(pre: FSAI, value_dtype=None, vector_dtype=None,
                 max_rhs=MAX_RHS) -> BatchedOperator:
    g, gt = pre.G, pre.GT
    if g.scalar_type == torch.bfloat16:
        raise ValueError("build the FSAI in float32 or float64; narrow with value_dtype")
    value_dtype = value_dtype or g.scalar_type
    vector_dtype = vector_dtype or (torch.float64 if value_dtype == torch.float64 else torch.float32)
    return _new("gbpc_bop_fsai", g.nrow, _lib.ptr(g.offsets), _lib.ptr(g.columns),
                _lib.ptr(g.values), _lib.ptr(gt.offsets), _lib.ptr(gt.columns),
                _lib.ptr(gt.values), _lib.dtype_code(g.scalar_type), _lib.dtype_code(value_dtype),
                _lib.dtype_code(vector_dtype), _max_rhs(max_rhs), _lib.stream(g.device),
                rows=g.nrow, vdt=vector_dtype, device=g.device, max_rhs=max_rhs)


def batched_sqlap(L: BsrMatrix, mass: torch.Tensor, mass_weight: float, value_dtype=torch.float64,
                  vector_dtype=None, max_rhs=MAX_RHS) -> BatchedOperator:
    """Factored ``mass_weight * M + L M^-1 L`` with every vertex free."""
    if L.scalar_type != torch.float64 or mass.dtype != torch.float64:
        raise TypeError("pass float64 L and mass; value_dtype selects the stored precision")
    vector_dtype = vector_dtype or (torch.float64 if value_dtype == torch.float64 else torch.float32)
    return _new("gbpc_bop_sqlap", L.nrow, _lib.ptr(L.offsets), _lib.ptr(L.columns),
                _lib.ptr(L.values), _lib.GBPC_F64, _lib.dtype_code(value_dtype),
                _lib.dtype_code(vector_dtype), _lib.ptr(mass.contiguous()), float(mass_weight),
                _max_rhs(max_rhs), _lib.stream(L.device), rows=L.nrow, vdt=vector_dtype,
                device=L.device, max_rhs=max_rhs)


class BatchedCG:
    """k independent PCG recurrences on one operator, per-RHS stopping."""

    def __init__(self, A: BatchedOperator, M: BatchedOperator, unroll=0, max_rhs=None):
        # M may be float32 behind a float64 A (float32-applied preconditioner).
        self.A, self.M = A, M
        self.max_rhs = _max_rhs(max_rhs if max_rhs is not None else min(A.max_rhs, M.max_rhs))
        out = ctypes.c_void_p()
        _lib.call("gbpc_bsolver_create", A._h, M._h, int(unroll), self.max_rhs,
                  _lib.stream(A.device), ctypes.byref(out))
        self._h = out
        self.nit = torch.zeros(MAX_RHS, dtype=torch.int32, device=A.device)
        self.rr = torch.zeros(MAX_RHS, dtype=torch.float64, device=A.device)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib._lib is not None:
            try:
                _lib._lib.gbpc_bsolver_destroy(h)
            except Exception:
                pass

    @property
    def device_bytes(self) -> int:
        return _lib.object_bytes("gbpc_bsolver_device_bytes", self._h)

    def run(self, B, X, tol=1e-8, atol=0.0, maxiter=0):
        k = _check_block(B, self.A.rows, self.A.dtype, self.max_rhs)
        _check_block(X, self.A.rows, self.A.dtype, self.max_rhs)
        _lib.call("gbpc_bsolver_run", self._h, k, _lib.ptr(B), _lib.ptr(X), float(tol),
                  float(atol), int(maxiter), _lib.ptr(self.nit), _lib.ptr(self.rr),
                  _lib.stream(self.A.device))
        return self.nit[:k], self.rr[:k]


def refine(A64: BatchedOperator, inner: BatchedCG, B, X, tol_outer=1e-12, tol_inner=1e-3,
           max_outer=20, max_inner=0):
    """Float64 iterative refinement around `inner`; returns (outer, inner) counts per RHS."""
    k = _check_block(B, A64.rows, torch.float64)
    _check_block(X, A64.rows, torch.float64)
    outer = (ctypes.c_int32 * k)()
    inner_it = (ctypes.c_int32 * k)()
    _lib.call("gbpc_refine", A64._h, inner._h, k, _lib.ptr(B), _lib.ptr(X), float(tol_outer),
              float(tol_inner), int(max_outer), int(max_inner), outer, inner_it,
              _lib.stream(A64.device))
    return list(outer), list(inner_it)


class BatchedSolver:
    """k right-hand sides of the factored smoothing system in one float64
    batched PCG (float64 operator and vectors; `factor_dtype` stores the FSAI
    factor).  Matrix bytes are read once per iteration for the whole batch.

    ``apply_dtype=torch.float32`` applies the preconditioner with float32
    arithmetic (factor stored in ``factor_dtype``, float32 or bfloat16): the
    update kernel hands it a float32 copy of the residual and the direction
    update widens its output, while the operator, the recurrences and every
    dot product stay float64."""

    def __init__(self, L: BsrMatrix, mass: torch.Tensor, mass_weight: float, pre: FSAI,
                 factor_dtype=torch.float64, unroll=0, apply_dtype=None):
        self.A = batched_sqlap(L, mass, mass_weight, torch.float64, torch.float64)
        if apply_dtype == torch.float32:
            if factor_dtype not in (torch.float32, torch.bfloat16):
                raise ValueError("a float32 apply needs float32 or bfloat16 factor storage")
            self.M = batched_fsai(pre, factor_dtype, torch.float32)
        elif apply_dtype in (None, torch.float64):
            self.M = batched_fsai(pre, factor_dtype, torch.float64)
        else:
            raise ValueError("apply_dtype must be torch.float64 or torch.float32")
        self.cg = BatchedCG(self.A, self.M, unroll)

    def solve(self, B, X, tol=1e-8, atol=0.0, maxiter=0):
        return self.cg.run(B, X, tol, atol, maxiter)


class MixedPrecisionSolver:
    """Float32 inner PCG with float64 refinement for the factored smoothing operator.

    ``factor_dtype`` is the storage of the FSAI factor in the inner solve
    (float32 or bfloat16); the operator is stored in float32 for the inner
    solve and float64 for the residual.
    """

    def __init__(self, L: BsrMatrix, mass: torch.Tensor, mass_weight: float, pre: FSAI,
                 factor_dtype=torch.bfloat16, unroll=0):
        self.A64 = batched_sqlap(L, mass, mass_weight, torch.float64, torch.float64)
        self.A32 = batched_sqlap(L, mass, mass_weight, torch.float32, torch.float32)
        self.M32 = batched_fsai(pre, factor_dtype, torch.float32)
        self.inner = BatchedCG(self.A32, self.M32, unroll)

    def solve(self, B, X, tol_outer=1e-12, tol_inner=1e-3, max_outer=20, max_inner=0):
        return refine(self.A64, self.inner, B, X, tol_outer, tol_inner, max_outer, max_inner)
