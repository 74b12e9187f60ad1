"""Block Jacobi and synchronous block ILU(0) (warp_preconditioners/block_ilu.py)."""

from __future__ import annotations

import math

import torch

from . import _lib
from .linear import LinearOperator
from .sparse import BsrMatrix


def _tolerance(A, pivot_tolerance):
    tol = (1e-12 if A.scalar_type == torch.float64 else 1e-6) if pivot_tolerance is None \
        else pivot_tolerance
    if not math.isfinite(tol) or tol < 0:
        raise ValueError("pivot_tolerance must be finite and nonnegative")
    return float(tol)


def _check_matrix(A):
    if not isinstance(A, BsrMatrix) or A.nrow != A.ncol:
        raise ValueError("A must be a square BSR matrix")
    size = A.block_shape[0]
    if A.block_shape != (size, size) or size not in (1, 2, 3, 4):
        raise ValueError("BlockJacobi requires square blocks of size 1 through 4")
    if A.scalar_type not in (torch.float32, torch.float64):
        raise TypeError("A must use float32 or float64")
    return size


class BlockJacobi(LinearOperator):
    """Invert diagonal 1x1..4x4 blocks on device; singular blocks raise.

    ``inverse_diagonal`` holds the inverse blocks, shape ``[nrow, b, b]``.
    ``update(A)`` recomputes them for new values; a failed update leaves the
    previous inverse in place.
    """

    def __init__(self, A, pivot_tolerance=None):
        size = _check_matrix(A)
        self.pivot_tolerance = _tolerance(A, pivot_tolerance)
        self.A = A
        self.block = size
        self.inverse_diagonal = torch.empty((A.nrow, size, size), dtype=A.scalar_type,
                                            device=A.device)
        self._op = self._build(A)
        super().__init__(A.shape, A.scalar_type, A.device, self._apply)

    def _build(self, A):
        inverse = torch.empty((A.nrow, self.block, self.block), dtype=A.scalar_type,
                              device=A.device)
        op = _lib.new_op("gbpc_op_block_jacobi", A.nrow, self.block, _lib.ptr(A.offsets),
                         _lib.ptr(A.columns), _lib.ptr(A.values), _lib.dtype_code(A.scalar_type),
                         self.pivot_tolerance, _lib.ptr(inverse), _lib.stream(A.device))
        self.inverse_diagonal = inverse
        return op

    def update(self, A=None):
        """Recompute diagonal inverses; a failed update keeps the previous ones."""
        if type(self) is not BlockJacobi:
            raise NotImplementedError("Rebuild BlockILU0 to update its factors")
        A = self.A if A is None else A
        if not isinstance(A, BsrMatrix) or (A.shape, A.scalar_type, A.device) != (
            self.shape, self.dtype, self.device,
        ):
            raise ValueError("update requires the same shape, dtype, and device")
        # In place (the operator's inverse and inverse_diagonal keep their
        # storage, so captured applies see the new values); a failed update
        # changes nothing.
        _lib.call("gbpc_op_block_jacobi_update", self._op.handle, A.nrow, self.block,
                  _lib.ptr(A.offsets), _lib.ptr(A.columns), _lib.ptr(A.values),
                  _lib.dtype_code(A.scalar_type), self.pivot_tolerance,
                  _lib.ptr(self.inverse_diagonal), _lib.stream(A.device))
        self.A = A
        return self

    def _apply(self, x, y, z, alpha, beta):
        self._op.apply(x.reshape(-1), y.reshape(-1) if y is not None else None, z.view(-1),
                       alpha, beta, self.device)


class BlockILU0(BlockJacobi):
    """Synchronous block ILU(0) with ``factor_sweeps`` setup sweeps and
    ``solve_sweeps`` Jacobi triangular sweeps per apply.

    ``factors`` holds the L/U blocks in A's block order (unit-diagonal L
    implied), ``inverse_diagonal`` the inverses of U's diagonal blocks.  The
    result is linear but generally nonsymmetric.
    """

    def __init__(self, A, factor_sweeps=12, solve_sweeps=4, relaxation=1.0, pivot_tolerance=None):
        if isinstance(factor_sweeps, bool) or not isinstance(factor_sweeps, int) \
                or factor_sweeps < 0:
            raise ValueError("factor_sweeps must be a nonnegative integer")
        if isinstance(solve_sweeps, bool) or not isinstance(solve_sweeps, int) or solve_sweeps < 1:
            raise ValueError("solve_sweeps must be a positive integer")
        if not math.isfinite(relaxation) or not 0 < relaxation <= 1:
            raise ValueError("relaxation must be in (0,1]")
        size = _check_matrix(A)
        self.pivot_tolerance = _tolerance(A, pivot_tolerance)
        self.A = A
        self.block = size
        self.factor_sweeps, self.solve_sweeps = factor_sweeps, solve_sweeps
        self.relaxation = float(relaxation)
        self.factors = torch.empty((A.nnz, size, size), dtype=A.scalar_type, device=A.device)
        self.inverse_diagonal = torch.empty((A.nrow, size, size), dtype=A.scalar_type,
                                            device=A.device)
        self._op = _lib.new_op(
            "gbpc_op_bilu0", A.nrow, size, _lib.ptr(A.offsets), _lib.ptr(A.columns),
            _lib.ptr(A.values), _lib.dtype_code(A.scalar_type), factor_sweeps, solve_sweeps,
            self.relaxation, self.pivot_tolerance, _lib.ptr(self.factors),
            _lib.ptr(self.inverse_diagonal), _lib.stream(A.device))
        LinearOperator.__init__(self, A.shape, A.scalar_type, A.device, self._apply)
