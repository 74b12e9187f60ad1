"""Block-row adaptive FSAI (benchmarks/block_fsai_candidate.py).

``BlockFSAI`` builds G with whole b x b block rows: greedy block growth
(score = sum of squared residuals over the b x b candidate block), a full
local Cholesky per step, b right-hand sides, and the block-row
normalisation ``G = chol(Z_ii)^-1 Z^T D^-1/2``.  ``BsrBlockFSAI`` applies it
as native b x b block products (``B``, ``BT``) with float32 storage and
float64 accumulation.
"""

from __future__ import annotations

import torch

from . import _lib
from .fsai import convert_factor, pack_rows
from .linear import LinearOperator
from .sparse import BsrMatrix, bsr_transposed, to_blocks


class BlockFSAI(LinearOperator):
    def __init__(self, a, max_blocks=2, apply_lanes=1, factor_dtype=torch.float32,
                 reuse_pattern=False):
        if not isinstance(a, BsrMatrix):
            raise TypeError("BlockFSAI requires a BSR matrix")
        block = a.block_shape[0]
        if not (block == a.block_shape[1] and block > 1):
            raise ValueError("BlockFSAI requires square blocks larger than 1x1")
        if a.scalar_type != torch.float64:
            raise TypeError("BlockFSAI setup runs on float64 matrices")
        n, dt, dev = a.shape[0], a.scalar_type, a.device
        width = block * max_blocks
        self.block, self.max_blocks, self.width = block, max_blocks, width
        self.apply_lanes = apply_lanes
        self.factor_dtype = factor_dtype
        self.source = a
        cols = torch.empty(n * width, dtype=torch.int32, device=dev)
        vals = torch.empty(n * width, dtype=dt, device=dev)
        counts = torch.empty(n, dtype=torch.int32, device=dev)
        self.scale = torch.empty(n, dtype=dt, device=dev)
        _lib.call("gbpc_block_fsai_setup", a.nrow, block, max_blocks, _lib.ptr(a.offsets),
                  _lib.ptr(a.columns), _lib.ptr(a.values), 0, _lib.ptr(cols), _lib.ptr(vals),
                  _lib.ptr(counts), _lib.ptr(self.scale), _lib.stream(dev), what="BlockFSAI")
        self._ell = (cols, vals, counts) if reuse_pattern else None
        g = pack_rows(n, width, cols, vals, counts)
        if factor_dtype != dt:
            g = convert_factor(g, factor_dtype)
        self.G = g
        self.GT = bsr_transposed(g)
        self._op = self._make_op(self.G, self.GT, 1, dt)
        super().__init__(a.shape, dt, dev, self._apply)

    def _make_op(self, g, gt, block, dt):
        return _lib.new_op(
            "gbpc_op_fsai", g.nrow, block, _lib.ptr(g.offsets), _lib.ptr(g.columns),
            _lib.ptr(g.values), _lib.ptr(gt.offsets), _lib.ptr(gt.columns), _lib.ptr(gt.values),
            _lib.dtype_code(g.scalar_type), _lib.dtype_code(dt), _lib.stream(g.device))

    def _apply(self, x, y, z, alpha, beta):
        self._op.apply(x.reshape(-1), y.reshape(-1) if y is not None else None, z.view(-1),
                       alpha, beta, self.device)


class BsrBlockFSAI(BlockFSAI):
    """BlockFSAI applied through b x b block products of ``B = G`` and ``BT``."""

    def __init__(self, a, **kw):
        super().__init__(a, **kw)
        self.B = to_blocks(self.G, self.block)
        self.BT = bsr_transposed(self.B)
        self._op = self._make_op(self.B, self.BT, self.block, a.scalar_type)
