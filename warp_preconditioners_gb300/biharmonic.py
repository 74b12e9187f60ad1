"""Lifted first-order biharmonic system (warp_preconditioners/biharmonic.py).

``BiharmonicSystem(K, mass, tau)`` builds the interleaved 2 x 2-block matrix
``[[M, -sqrt(tau) K], [sqrt(tau) K, M]]`` and the SPD target
``H = M + sqrt(tau) K``; ``preconditioner(**fsai_options)`` returns
``RepeatedFSAI(FSAI(H))``, which applies the scalar FSAI to both components
of vec2 arrays through 2 x 2 block products of ``diag(G, G)``.  The lifted
system is nonsymmetric: solve it with ``linear.gmres`` (never CG/CR).
"""

from __future__ import annotations

import math

import torch

from . import _lib
from .fsai import FSAI
from .linear import LinearOperator
from .sparse import BsrMatrix, bsr_from_triplets, bsr_transposed


def _row_ids(a: BsrMatrix) -> torch.Tensor:
    counts = (a.offsets[1:] - a.offsets[:-1]).to(torch.int64)
    return torch.repeat_interleave(torch.arange(a.nrow, device=a.device), counts)


class RepeatedFSAI(LinearOperator):
    """Apply the same scalar FSAI independently to both components of vec2 arrays."""

    def __init__(self, factor: FSAI):
        self.factor = factor
        g = factor.G
        dt = g.scalar_type
        blocks = torch.zeros((g.nnz, 2, 2), dtype=dt, device=g.device)
        blocks[:, 0, 0] = g.values
        blocks[:, 1, 1] = g.values
        self.G = BsrMatrix(g.nrow, g.ncol, (2, 2), g.offsets, g.columns, blocks)
        self.GT = bsr_transposed(self.G)
        vdt = factor.dtype
        self._op = _lib.new_op(
            "gbpc_op_fsai", g.nrow, 2, _lib.ptr(self.G.offsets), _lib.ptr(self.G.columns),
            _lib.ptr(self.G.values), _lib.ptr(self.GT.offsets), _lib.ptr(self.GT.columns),
            _lib.ptr(self.GT.values), _lib.dtype_code(dt), _lib.dtype_code(vdt),
            _lib.stream(g.device))
        super().__init__((2 * g.nrow, 2 * g.ncol), vdt, g.device, self._apply)

    def _apply(self, x, y, z, alpha, beta):
        self._op.apply(x.reshape(-1), y.reshape(-1) if y is not None else None, z.view(-1),
                       alpha, beta, self.device)


class BiharmonicSystem:
    def __init__(self, K, mass, tau=1.0):
        if not isinstance(K, BsrMatrix) or K.shape[0] != K.shape[1] or K.block_shape != (1, 1):
            raise ValueError("K must be a square scalar BSR matrix")
        if K.scalar_type not in (torch.float32, torch.float64):
            raise TypeError("K must use float32 or float64")
        if mass.dtype != K.scalar_type or mass.device != K.device or tuple(mass.shape) != (K.nrow,):
            raise ValueError("mass must match K's scalar dtype, device, and row count")
        if not math.isfinite(tau) or tau <= 0:
            raise ValueError("tau must be finite and positive")
        if not bool(torch.all(torch.isfinite(mass) & (mass > 0))):
            raise ValueError("mass must contain finite positive entries")
        self.K, self.mass, self.tau = K, mass.clone(), float(tau)
        n = K.nrow
        root = math.sqrt(tau)
        rows = torch.cat([torch.arange(n, device=K.device), _row_ids(K)])
        cols = torch.cat([torch.arange(n, device=K.device), K.columns.to(torch.int64)])
        k = root * K.values
        dt = K.scalar_type
        blocks = torch.zeros((n + K.nnz, 2, 2), dtype=dt, device=K.device)
        blocks[:n, 0, 0] = mass
        blocks[:n, 1, 1] = mass
        blocks[n:, 0, 1] = -k
        blocks[n:, 1, 0] = k
        hvals = torch.cat([mass, k])
        self.matrix = bsr_from_triplets(n, n, rows, cols, blocks)
        self.H = bsr_from_triplets(n, n, rows, cols, hvals)

    def preconditioner(self, **fsai_options):
        return RepeatedFSAI(FSAI(self.H, **fsai_options))

    def rhs(self, b):
        """Embed a scalar RHS as interleaved (b, 0)."""
        if b.shape != self.mass.shape or b.dtype != self.mass.dtype or b.device != self.mass.device:
            raise ValueError("b must match mass's shape, dtype and device")
        out = torch.zeros((b.numel(), 2), dtype=b.dtype, device=b.device)
        out[:, 0] = b
        return out

    def solution(self, x, out=None):
        """Extract u from a lifted solution."""
        if x.dim() != 2 or x.shape != (self.mass.numel(), 2) or x.dtype != self.mass.dtype:
            raise ValueError("x must be a vec2 solution on the system device")
        if out is None:
            out = torch.empty_like(self.mass)
        if out.dtype != self.mass.dtype or out.shape != self.mass.shape:
            raise ValueError("out must match mass's shape, dtype and device")
        out.copy_(x[:, 0])
        return out
