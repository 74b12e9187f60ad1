"""Many independent systems of uneven size in one solve.

Two ways:

* ``ClusterSolver(systems)``: each (A, M) pair keeps its own operators;
  one launch gives every system its own thread-block cluster, which runs
  that system's whole PCG solve and leaves when it has converged (small
  systems: a float64 sparse or factored squared-Laplacian operator, an FSAI
  or no preconditioner).
* ``MultiSystemSolver(A, M, sizes)``, below.

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

__all__ = ["ClusterSolver", "MultiSystemSolver", "block_diag", "concat_vectors", "split_vector"]


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


class ClusterSolver:
    """PCG on many independent systems in one launch, one thread-block
    cluster per system (gbpc_csolver).  ``systems`` is a list of (A, M)
    pairs of library operators (M may be None).  A system's iterates equal
    those of the drop-in CG solver on that system alone below 32,768 rows
    (the same cluster kernel).  No reference counterpart."""

    def __init__(self, systems):
        systems = [(aslinearoperator(a), aslinearoperator(m)) for a, m in systems]
        if not systems:
            raise ValueError("ClusterSolver needs at least one system")
        self.systems = systems
        self.device = systems[0][0].device
        S = len(systems)
        A = (ctypes.c_void_p * S)(*[_handle(a) for a, _ in systems])
        M = (ctypes.c_void_p * S)(*[_handle(m) if m is not None else None for _, m in systems])
        out = ctypes.c_void_p()
        _lib.call("gbpc_csolver_create", S, A, M, _lib.stream(self.device), ctypes.byref(out))
        self._h = out
        self.nit = torch.zeros(S, dtype=torch.int32, device=self.device)
        self.rr = torch.zeros(S, dtype=torch.float64, device=self.device)
        self.atol_sq = torch.zeros(S, dtype=torch.float64, device=self.device)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib._lib is not None:
            try:
                _lib._lib.gbpc_csolver_destroy(h)
            except Exception:
                pass

    @property
    def cluster_size(self) -> int:
        c = ctypes.c_int()
        _lib.call("gbpc_csolver_cluster_size", self._h, ctypes.byref(c))
        return int(c.value)

    @property
    def device_bytes(self) -> int:
        return _lib.object_bytes("gbpc_csolver_device_bytes", self._h)

    def run(self, bs, xs, tol=None, atol=None, maxiter=0):
        """Solve system s for bs[s] from the initial guess xs[s] (float64
        device tensors) for the first len(bs) systems; returns device arrays
        (iterations, r.r, atol^2), one entry per system solved.
        Stream-ordered, no synchronisation."""
        S = len(bs)
        if not 1 <= S <= len(self.systems) or len(xs) != S:
            raise ValueError(f"expected 1..{len(self.systems)} right-hand sides and as many "
                             f"solution vectors")
        for (a, _), b, x in zip(self.systems[:S], bs, xs):
            if b.dtype != torch.float64 or x.dtype != torch.float64:
                raise TypeError("the cluster solver runs on float64 vectors")
            if b.numel() != a.shape[0] or x.numel() != a.shape[0]:
                raise ValueError("vector length differs from its system's size")
        tol = 1.0e-5 if tol is None else float(tol)
        atol = 0.0 if atol is None else float(atol)
        bp = (ctypes.c_void_p * S)(*[_lib.ptr(_flat(b)).value for b in bs])
        xp = (ctypes.c_void_p * S)(*[_lib.ptr(_flat(x)).value for x in xs])
        _lib.call("gbpc_csolver_run", self._h, S, bp, xp, tol, atol, int(maxiter),
                  _lib.ptr(self.nit), _lib.ptr(self.rr), _lib.ptr(self.atol_sq),
                  _lib.stream(self.device))
        return self.nit[:S], self.rr[:S], self.atol_sq[:S]
