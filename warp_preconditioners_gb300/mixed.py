"""Mixed harmonic (symmetric indefinite) systems and their block
preconditioners (warp_preconditioners/mixed.py).

``MixedHarmonicSystem(K, mass, order, data_weight, equilibrate)`` assembles
the interleaved 2- or 3-field block matrix of the reference benchmark, with
the reference's signs: order 2 ``[[alpha M, -K], [-K, -M]]``, order 3
``[[alpha M, 0, -K], [0, -K, -M], [-K, -M, 0]]``, and the SPD matrix
``H = K + alpha^(1/order) M``.  ``equilibrate=True`` builds ``D A D`` with
``D = (alpha^-1/4, alpha^1/4)`` (order 2) or ``(alpha^-1/3, 1, alpha^1/3)``
(order 3); ``rhs``, ``transform`` and ``solution`` apply the matching change
of variables.  These systems are nonsymmetric-indefinite territory: solve
them with ``linear.gmres``.

``MatchingSchur`` and ``ShiftedBlock`` are operators of libgbpc built on an
approximate ``H^-1`` (``FSAI(H)`` by default, or any operator of this
package), so a GMRES graph captures their whole apply.
"""

from __future__ import annotations

import math

import torch

from . import _lib
from .fsai import FSAI
from .linear import LinearOperator
from .sparse import BsrMatrix, bsr_from_triplets


def _row_ids(a: BsrMatrix) -> torch.Tensor:
    counts = (a.offsets[1:] - a.offsets[:-1]).to(torch.int64)
    return torch.repeat_interleave(torch.arange(a.nrow, device=a.device), counts)


class MixedHarmonicSystem:
    """The reference's symmetric indefinite 2/3-field systems (mixed.py:161-280)."""

    def __init__(self, K, mass, order=2, data_weight=1.0, equilibrate=False):
        if not isinstance(K, BsrMatrix) or K.nrow != K.ncol or K.block_shape != (1, 1):
            raise ValueError("K must be square scalar BSR")
        if K.scalar_type not in (torch.float32, torch.float64):
            raise TypeError("K must use float32 or float64")
        if mass.dtype != K.scalar_type or mass.device != K.device or tuple(mass.shape) != (K.nrow,):
            raise ValueError("mass must match K")
        if order not in (2, 3) or not math.isfinite(data_weight) or data_weight <= 0:
            raise ValueError("order must be 2 or 3 and data_weight finite positive")
        self.K = K
        self.mass = mass.clone().contiguous()
        self.order, self.data_weight = order, float(data_weight)
        self.input_data_weight = float(data_weight)
        self.equilibrate = bool(equilibrate)
        self.scale = (1.0,) * order
        if equilibrate:
            root = data_weight ** (1 / order)
            self.scale = ((data_weight ** -0.25, data_weight ** 0.25) if order == 2
                          else (1 / root, 1.0, root))
            self.mass = (root * mass).contiguous()
            self.data_weight = 1.0
        weight = self.data_weight
        shift = self.data_weight ** (1 / order)
        m = self.mass
        if not bool(torch.all(torch.isfinite(m) & (m > 0))):
            raise ValueError("mass must be finite positive")
        n, dev, dt = K.nrow, K.device, K.scalar_type
        rows = torch.cat([torch.arange(n, device=dev), _row_ids(K)])
        cols = torch.cat([torch.arange(n, device=dev), K.columns.to(torch.int64)])
        blocks = torch.zeros((n + K.nnz, order, order), dtype=dt, device=dev)
        v = K.values
        blocks[:n, 0, 0] = weight * m
        if order == 2:
            blocks[:n, 1, 1] = -m
            blocks[n:, 0, 1] = -v
            blocks[n:, 1, 0] = -v
        else:
            blocks[:n, 1, 2] = -m
            blocks[:n, 2, 1] = -m
            blocks[n:, 0, 2] = -v
            blocks[n:, 2, 0] = -v
            blocks[n:, 1, 1] = -v
        hvalues = torch.cat([shift * m, v])
        self.matrix = bsr_from_triplets(n, n, rows, cols, blocks)
        self.H = bsr_from_triplets(n, n, rows, cols, hvalues)
        self._scale_t = torch.tensor(self.scale, dtype=dt, device=dev)

    def rhs(self, b):
        """Interleaved (b, 0[, 0]), transformed when equilibrated."""
        if b.dtype != self.mass.dtype or b.shape != self.mass.shape or b.device != self.mass.device:
            raise ValueError("b must match mass")
        out = torch.zeros((self.K.nrow, self.order), dtype=b.dtype, device=b.device)
        out[:, 0] = b
        if self.equilibrate:
            self.transform(out, out)
        return out

    def transform(self, x, out=None):
        """Apply D: maps original RHS to balanced RHS, or balanced solution to original."""
        if (x.dim() != 2 or tuple(x.shape) != (self.K.nrow, self.order)
                or x.dtype != self.mass.dtype or x.device != self.mass.device):
            raise ValueError("x must be an interleaved system vector")
        if out is None:
            out = torch.empty_like(x)
        if out.dtype != x.dtype or out.shape != x.shape or out.device != x.device:
            raise ValueError("out must match x")
        torch.mul(x, self._scale_t, out=out)
        return out

    def solution(self, x):
        if (x.dim() != 2 or tuple(x.shape) != (self.K.nrow, self.order)
                or x.dtype != self.mass.dtype or x.device != self.mass.device):
            raise ValueError("x must be an interleaved system vector")
        if self.equilibrate:
            x = self.transform(x)
        return x[:, 0].clone()


def _inverse_for(system, H_inverse, fsai_options):
    inverse = FSAI(system.H, **fsai_options) if H_inverse is None else H_inverse
    if (tuple(inverse.shape) != tuple(system.H.shape) or inverse.dtype != system.H.dtype
            or inverse.device != system.H.device):
        raise ValueError("H_inverse must match H")
    if getattr(inverse, "_op", None) is None:
        raise TypeError("H_inverse must be an operator of this package (FSAI, SparseOperator, "
                        "BlockJacobi, ...)")
    return inverse


class MatchingSchur(LinearOperator):
    """Block elimination using repeated approximate inverses of H (mixed.py:283-334).

    The Schur inverse approximation is ``H^-1 M H^-1`` for order 2 and
    ``-H^-1 M H^-1 M H^-1`` for the benchmark's order-3 signs; no inner
    adaptive solve is hidden, so ordinary right GMRES is valid.
    """

    def __init__(self, system, H_inverse=None, **fsai_options):
        self.system = system
        self.inverse = _inverse_for(system, H_inverse, fsai_options)
        K = system.K
        self._op = _lib.new_op("gbpc_op_matching_schur", system.order, K.nrow, _lib.ptr(K.offsets),
                               _lib.ptr(K.columns), _lib.ptr(K.values),
                               _lib.dtype_code(K.scalar_type), _lib.ptr(system.mass),
                               self.inverse._op.handle, _lib.stream(K.device))
        super().__init__(system.matrix.shape, K.scalar_type, K.device, self._apply)

    def _apply(self, x, y, z, alpha, beta):
        self._op.apply(x.reshape(-1), y.reshape(-1) if y is not None else None, z.view(-1),
                       alpha, beta, self.device)


class ShiftedBlock(LinearOperator):
    """First-order block approximation using H (mixed.py:388-427).

    Order 2 uses the balanced block rotation with ``scale = data_weight^(1/4)``;
    order 3 approximates the inverse of the leading K blocks.
    """

    def __init__(self, system, H_inverse=None, **fsai_options):
        self.system = system
        self.inverse = _inverse_for(system, H_inverse, fsai_options)
        K = system.K
        scale = system.data_weight ** 0.25
        self._op = _lib.new_op("gbpc_op_shifted_block", system.order, K.nrow, float(scale),
                               _lib.dtype_code(K.scalar_type), self.inverse._op.handle,
                               _lib.stream(K.device))
        super().__init__(system.matrix.shape, K.scalar_type, K.device, self._apply)

    def _apply(self, x, y, z, alpha, beta):
        self._op.apply(x.reshape(-1), y.reshape(-1) if y is not None else None, z.view(-1),
                       alpha, beta, self.device)
