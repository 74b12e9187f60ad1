"""Many independent systems of uneven size in one solve.

``MultiSystemSolver(A, M, sizes)`` runs preconditioned CG on S systems at
once: ``A`` and ``M`` are operators over the concatenated vectors whose
diagonal blocks are the systems (``sparse.block_diag`` of the system
matrices, a squared-Laplacian operator over concatenated meshes, FSAI of
the block-diagonal matrix), and ``sizes[s]`` is system s's number of
unknowns.  Every product is one launch for all systems; step lengths, dot
products, stopping tests and iteration counts are per system, and a
system's iterates do not depend on which other systems share the solve.
No reference counterpart: the reference solves one system per cg call.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .linear import _flat, _handle, aslinearoperator
from .sparse import block_diag

__all__ = ["MultiSystemSolver", "block_diag", "concat_vectors", "split_vector"]


class MultiSystemSolver:
    def __init__(self, A, M, sizes, use_cuda_graph=True, unroll=4):
        sizes = [int(s) for s in sizes]
        if not sizes or min(sizes) < 0:
            raise ValueError("sizes must be a non-empty list of non-negative row counts")
        self.A = aslinearoperator(A)
        self.M = aslinearoperator(M)
        self.sizes = sizes
        self.offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        if int(self.offsets[-1]) != self.A.shape[0]:
            raise ValueError(f"sizes add up to {int(self.offsets[-1])}, the operator has "
                             f"{self.A.shape[0]} rows")
        out = ctypes.c_void_p()
        _lib.call("gbpc_msolver_create", _handle(self.A), _handle(self.M), len(sizes),
                  self.offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                  int(bool(use_cuda_graph)), int(unroll), _lib.stream(self.A.device),
                  ctypes.byref(out))
        self._h = out
        dev = self.A.device
        self.nit = torch.zeros(len(sizes), dtype=torch.int32, device=dev)
        self.rr = torch.zeros(len(sizes), dtype=torch.float64, device=dev)
        self.atol_sq = torch.zeros(len(sizes), dtype=torch.float64, device=dev)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib._lib is not None:
            try:
                _lib._lib.gbpc_msolver_destroy(h)
            except Exception:
                pass

    @property
    def device_bytes(self) -> int:
        return _lib.object_bytes("gbpc_msolver_device_bytes", self._h)

    def run(self, b, x, tol=None, atol=None, maxiter=0):
        """Solve every system to its own stopping test (r_s.r_s <= max(atol,
        tol |b_s|)^2, or maxiter iterations; maxiter <= 0 means the system's
        size).  Returns device arrays (iterations, r.r, atol^2), one entry
        per system.  Stream-ordered, no synchronisation."""
        if b.dtype != torch.float64 or x.dtype != torch.float64:
            raise TypeError("the multi-system solver runs on float64 vectors")
        tol = 1.0e-5 if tol is None else float(tol)
        atol = 0.0 if atol is None else float(atol)
        _lib.call("gbpc_msolver_run", self._h, _lib.ptr(_flat(b)), _lib.ptr(_flat(x)), tol, atol,
                  int(maxiter), _lib.ptr(self.nit), _lib.ptr(self.rr), _lib.ptr(self.atol_sq),
                  _lib.stream(self.A.device))
        return self.nit, self.rr, self.atol_sq


def concat_vectors(vs) -> torch.Tensor:
    """Concatenate per-system vectors into the solver's layout."""
    return torch.cat([v.reshape(-1) for v in vs]).contiguous()


def split_vector(x, sizes) -> list:
    """Per-system views of a concatenated vector."""
    return list(torch.split(x, [int(s) for s in sizes]))
