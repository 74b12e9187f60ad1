"""Factored squared Laplacian (warp_preconditioners/squared_laplacian.py).

Applies ``(L diag(1/mass) L + mass_weight diag(mass))[free, free]`` through
two sparse products with L instead of an assembled ``K M^-1 K``: a forward
product over all rows of L into ``tmp = M^-1 L R x`` and a backward product
over the free rows with the mass term fused into its epilogue.
"""

from __future__ import annotations

import math

import torch

from . import _lib
from .linear import LinearOperator
from .sparse import BsrMatrix


class SquaredLaplacianOperator(LinearOperator):
    def __init__(self, L, mass, free_indices, row_lanes=1, mass_weight=0.0):
        if not isinstance(L, BsrMatrix) or L.nrow != L.ncol or L.block_shape != (1, 1):
            raise ValueError("L must be a square scalar BSR matrix")
        if L.scalar_type not in (torch.float32, torch.float64):
            raise TypeError("L must use float32 or float64")
        if mass.device != L.device or free_indices.device != L.device:
            raise ValueError("L, mass, and free_indices must be on the same device")
        if mass.dtype != L.scalar_type or mass.dim() != 1 or mass.numel() != L.nrow:
            raise ValueError("mass must match the scalar type and size of L")
        if free_indices.dtype != torch.int32 or free_indices.dim() != 1:
            raise ValueError("free_indices must be a one-dimensional int32 array")
        if not isinstance(row_lanes, int) or row_lanes not in (1, 2, 4, 8, 16, 32):
            raise ValueError("row_lanes must be one of 1, 2, 4, 8, 16, 32")
        if not math.isfinite(mass_weight) or mass_weight < 0:
            raise ValueError("mass_weight must be finite and nonnegative")
        self.mass_weight = float(mass_weight)
        self.L = L
        self.mass = mass.contiguous()
        self.free = free_indices.clone().contiguous()
        self.row_lanes = row_lanes
        self._op = _lib.new_op(
            "gbpc_op_sqlap", L.nrow, _lib.ptr(L.offsets), _lib.ptr(L.columns), _lib.ptr(L.values),
            _lib.dtype_code(L.scalar_type), _lib.ptr(self.mass), _lib.ptr(self.free),
            int(self.free.numel()), self.mass_weight, _lib.stream(L.device),
            what="SquaredLaplacianOperator")
        n = int(self.free.numel())
        super().__init__((n, n), L.scalar_type, L.device, self._apply)

    def _apply(self, x, y, z, alpha, beta):
        self._op.apply(x.reshape(-1), y.reshape(-1) if y is not None else None, z.view(-1),
                       alpha, beta, self.device)

    def rhs(self, boundary_values, out=None):
        """Eliminated right-hand side ``-(Q u_b)[free]`` (squared_laplacian.py:200-218)."""
        if (boundary_values.dtype != self.scalar_type or boundary_values.device != self.device
                or boundary_values.dim() != 1 or boundary_values.numel() != self.L.nrow):
            raise ValueError("boundary_values must match the scalar type, device, and size of L")
        n = int(self.free.numel())
        if out is None:
            out = torch.empty(n, dtype=self.scalar_type, device=self.device)
        elif (out.dtype != self.scalar_type or out.device != self.device or out.dim() != 1
              or out.numel() != n):
            raise ValueError("out must match the reduced operator")
        _lib.call("gbpc_sqlap_rhs", self._op.handle, _lib.ptr(boundary_values.contiguous()),
                  _lib.ptr(out), _lib.stream(self.device))
        return out
