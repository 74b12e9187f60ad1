"""Sparse product operator (warp_preconditioners/sparse_operator.py).

``SparseOperator(A, row_lanes=4)`` applies ``z = alpha * A x + beta * y`` with
the library's sliced-ELL product (one thread per row; the reference's
``row_lanes`` cooperative grouping is validated and recorded, since on GB300
full-lane FP64 issue favours one thread per row).  x may alias z: the operator
then copies x to scratch first, as the reference does.
"""

from __future__ import annotations

import torch

from . import _lib
from .linear import LinearOperator
from .sparse import BsrMatrix


class SparseOperator(LinearOperator):
    def __init__(self, A, row_lanes=4):
        if not isinstance(A, BsrMatrix):
            raise TypeError("SparseOperator requires a BSR matrix")
        if A.scalar_type not in (torch.float32, torch.float64):
            raise TypeError("SparseOperator supports float32 and float64")
        if not isinstance(row_lanes, int) or row_lanes not in (1, 2, 4, 8, 16, 32):
            raise ValueError("row_lanes must be one of 1, 2, 4, 8, 16, 32")
        self.source = A
        self.row_lanes = row_lanes
        b = A.block_shape[0]
        dt = A.scalar_type
        self._op = _lib.new_op("gbpc_op_sparse", A.nrow, A.ncol, b, _lib.ptr(A.offsets),
                               _lib.ptr(A.columns), _lib.ptr(A.values), _lib.dtype_code(dt),
                               _lib.dtype_code(dt), _lib.stream(A.device))
        super().__init__(A.shape, dt, A.device, self._apply)

    def _apply(self, x, y, z, alpha, beta):
        self._op.apply(x.reshape(-1), y.reshape(-1) if y is not None else None, z.view(-1),
                       alpha, beta, self.device)
