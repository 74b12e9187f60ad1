"""LinearOperator protocol and the CG / CR entry points.

Mirrors the parts of ``warp.optim.linear`` that the reference uses: the
``LinearOperator(shape, dtype, device, matvec)`` base with
``matvec(x, y, z, alpha, beta)`` computing ``z = alpha * Op x + beta * y``,
``aslinearoperator``, ``preconditioner(A, "diag")`` and ``cg`` / ``cr`` /
``gmres`` with the same signatures and return values (device arrays when
``check_every=0``).  The loops themselves run in libgbpc (one CUDA graph per
solve).
"""

from __future__ import annotations

import contextlib
import ctypes
import math
import threading

import torch

from . import _lib
from .sparse import BsrMatrix


class LinearOperator:
    def __init__(self, shape, dtype, device, matvec):
        self.shape = tuple(shape)
        self.dtype = dtype
        self.device = torch.device(device)
        self._matvec = matvec

    @property
    def scalar_type(self) -> torch.dtype:
        return self.dtype

    def matvec(self, x, y, z, alpha, beta):
        self._matvec(x, y, z, alpha, beta)

    # Subclasses backed by libgbpc set `_op` (an _lib.OpHandle).
    _op = None


class _HandleOperator(LinearOperator):
    """A LinearOperator whose apply is one libgbpc operator."""

    def __init__(self, handle: _lib.OpHandle, shape, dtype, device):
        self._op = handle
        super().__init__(shape, dtype, device, self._apply)

    def _apply(self, x, y, z, alpha, beta):
        self._op.apply(_flat(x), _flat(y) if y is not None else None, _flat(z), alpha, beta,
                       self.device)


def _flat(t: torch.Tensor) -> torch.Tensor:
    if not t.is_contiguous():
        raise ValueError("vectors must be contiguous")
    return t.view(-1)


def aslinearoperator(a) -> LinearOperator | None:
    """BsrMatrix -> sparse-product operator; LinearOperators pass through."""
    if a is None or isinstance(a, LinearOperator):
        return a
    if isinstance(a, BsrMatrix):
        cached = getattr(a, "_gbpc_linop", None)
        if cached is not None:
            return cached
        b = a.block_shape[0]
        dt = a.scalar_type
        h = _lib.new_op("gbpc_op_sparse", a.nrow, a.ncol, b, _lib.ptr(a.offsets),
                        _lib.ptr(a.columns), _lib.ptr(a.values), _lib.dtype_code(dt),
                        _lib.dtype_code(dt), _lib.stream(a.device))
        op = _HandleOperator(h, a.shape, dt, a.device)
        a._gbpc_linop = op
        return op
    raise TypeError(f"cannot make a linear operator from {type(a).__name__}")


def preconditioner(A, ptype="diag") -> LinearOperator:
    """Scalar Jacobi preconditioner on the scalar diagonal of A."""
    if ptype != "diag":
        raise ValueError(f"unsupported preconditioner type {ptype!r}")
    if not isinstance(A, BsrMatrix):
        raise TypeError("preconditioner() needs a BsrMatrix")
    b = A.block_shape[0]
    h = _lib.new_op("gbpc_op_diagonal", A.nrow, b, _lib.ptr(A.offsets), _lib.ptr(A.columns),
                    _lib.ptr(A.values), _lib.dtype_code(A.scalar_type), _lib.stream(A.device))
    return _HandleOperator(h, A.shape, A.scalar_type, A.device)


def _handle(op: LinearOperator | None):
    if op is None:
        return None
    h = getattr(op, "_op", None)
    if h is None:
        raise TypeError(f"{type(op).__name__} has no libgbpc operator")
    return h.handle


class Solver:
    """Reusable CG / CR solver bound to (A, M); repeated runs replay one graph."""

    def __init__(self, method: str, A, M=None, use_cuda_graph=True, unroll=0):
        self.A = aslinearoperator(A)
        self.M = aslinearoperator(M)
        code = _lib.GBPC_CG if method == "cg" else _lib.GBPC_CR
        out = ctypes.c_void_p()
        _lib.call("gbpc_solver_create", code, _handle(self.A), _handle(self.M),
                  int(bool(use_cuda_graph)), int(unroll), _lib.stream(self.A.device),
                  ctypes.byref(out))
        self._h = out
        dev = self.A.device
        self.nit = torch.zeros(1, dtype=torch.int32, device=dev)
        self.rr = torch.zeros(1, dtype=torch.float64, device=dev)
        self.atol_sq = torch.zeros(1, dtype=torch.float64, device=dev)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.load().gbpc_solver_destroy(h)
            except Exception:
                pass

    @property
    def device_bytes(self) -> int:
        """Device bytes of the Krylov state (work vectors and scalars)."""
        return _lib.object_bytes("gbpc_solver_device_bytes", self._h)

    @property
    def cluster_size(self) -> int:
        """CTAs of the thread-block cluster that runs the whole solve as one
        kernel (small systems), 0 when the graph loop of separate kernels
        runs it."""
        c = ctypes.c_int()
        _lib.call("gbpc_solver_cluster", self._h, ctypes.byref(c))
        return int(c.value)

    def run(self, b, x, tol=None, atol=None, maxiter=0, history=None):
        """Solve from the initial guess in x.  ``history`` (float64 device
        tensor, optional) receives |r_k| for k < len(history), k = 0 the
        initial residual; the iterates are the same with or without it."""
        tol = 1.0e-5 if tol is None else float(tol)
        atol = 0.0 if atol is None else float(atol)
        if history is not None:
            if history.dtype != torch.float64 or not history.is_cuda:
                raise TypeError("history must be a float64 CUDA tensor")
            _lib.call("gbpc_solver_set_history", self._h, _lib.ptr(_flat(history)),
                      int(history.numel()))
        else:
            _lib.call("gbpc_solver_set_history", self._h, None, 0)
        _lib.call("gbpc_solver_run", self._h, _lib.ptr(_flat(b)), _lib.ptr(_flat(x)), tol, atol,
                  int(maxiter), _lib.ptr(self.nit), _lib.ptr(self.rr), _lib.ptr(self.atol_sq),
                  _lib.stream(self.A.device))
        return self.nit, self.rr, self.atol_sq


class _Vec:
    """libgbpc vector kernels on flat device vectors of one dtype."""

    def __init__(self, n, dtype, device):
        self.n = n
        self.code = _lib.dtype_code(dtype)
        self.stream = _lib.stream(device)
        self.work = torch.empty(_lib.load().gbpc_vec_dot_work_size(), dtype=torch.float64,
                                device=device)
        self.out = torch.zeros(4, dtype=torch.float64, device=device)

    def axpby(self, alpha, x, beta, y, z):
        _lib.call("gbpc_vec_axpby", self.n, self.code, float(alpha),
                  _lib.ptr(x) if alpha != 0.0 else None, float(beta),
                  _lib.ptr(y) if beta != 0.0 else None, _lib.ptr(z), self.stream)

    def dot(self, x, y, slot):
        _lib.call("gbpc_vec_dot", self.n, self.code, _lib.ptr(x), _lib.ptr(y),
                  _lib.ptr(self.work), ctypes.c_void_p(self.out.data_ptr() + 8 * slot),
                  self.stream)

    def read(self, count):
        return self.out[:count].tolist()


def _host_krylov(method, A, M, b, x, tol, atol, maxiter, history=None):
    """CG / CR stepped from the host, for operators without a libgbpc handle
    (any ``LinearOperator(shape, dtype, device, matvec)``) and for float32
    systems.  Every vector update and dot product runs in libgbpc kernels on
    the device; the host reads the dot products (two synchronisations per
    iteration) to form the scalars.  Same recurrences and stopping rule as
    the device loop (warp.optim.linear: r.r <= max(atol, tol |b|)^2 or
    maxiter); float64 dot accumulation for every vector dtype."""
    bf, xf = _flat(b), _flat(x)
    n = bf.numel()
    dev = bf.device
    v = _Vec(n, bf.dtype, dev)
    r, z, p, Ap = (torch.empty_like(bf) for _ in range(4))

    def apply(op, src, dst):
        op.matvec(src.view(b.shape), dst.view(b.shape), dst.view(b.shape), 1.0, 0.0)

    def precondition(src, dst):
        if M is None:
            v.axpby(1.0, src, 0.0, None, dst)
        else:
            apply(M, src, dst)

    if maxiter <= 0:
        maxiter = n
    A.matvec(x, b, r.view(b.shape), -1.0, 1.0)  # r = b - A x
    v.dot(bf, bf, 0)
    v.dot(r, r, 1)
    precondition(r, z)
    v.axpby(1.0, z, 0.0, None, p)
    if method == "cg":
        v.dot(r, z, 2)
        bb, rr, rz = v.read(3)
    else:
        Az, y = torch.empty_like(bf), torch.empty_like(bf)
        apply(A, z, Az)
        v.axpby(1.0, Az, 0.0, None, Ap)
        v.dot(z, Az, 2)
        bb, rr, rz = v.read(3)
    atol_sq = max(atol, tol * math.sqrt(bb)) ** 2
    it = 0
    if history is not None:
        history.append(math.sqrt(max(rr, 0.0)))
    while rr > atol_sq and it < maxiter:
        if method == "cg":
            apply(A, p, Ap)
            v.dot(p, Ap, 0)
            (pap,) = v.read(1)
            alpha = rz / pap
            v.axpby(alpha, p, 1.0, xf, xf)
            v.axpby(-alpha, Ap, 1.0, r, r)
            precondition(r, z)
            v.dot(r, r, 0)
            v.dot(r, z, 1)
            rr, rz_new = v.read(2)
            beta = rz_new / rz
            rz = rz_new
            v.axpby(1.0, z, beta, p, p)
        else:
            precondition(Ap, y)
            v.dot(Ap, y, 0)
            (apy,) = v.read(1)
            alpha = rz / apy
            v.axpby(alpha, p, 1.0, xf, xf)
            v.axpby(-alpha, Ap, 1.0, r, r)
            v.axpby(-alpha, y, 1.0, z, z)
            apply(A, z, Az)
            v.dot(r, r, 0)
            v.dot(z, Az, 1)
            rr, rz_new = v.read(2)
            beta = rz_new / rz
            rz = rz_new
            v.axpby(1.0, z, beta, p, p)
            v.axpby(1.0, Az, beta, Ap, Ap)
        it += 1
        if history is not None:
            history.append(math.sqrt(max(rr, 0.0)))
    return it, rr, atol_sq


_sampler = threading.local()


@contextlib.contextmanager
def sample_iterations(checkpoints, observe):
    """Observe the residual norm of every cg / cr call inside the block at
    iteration 0 and at each checkpoint (and where the solve stops early):
    ``observe(i, |r_i|)``.  The solves run as they would without it -- same
    iterates -- recording |r_k| in a device history buffer that is read
    once the solve ends (the reference's benchmarks/residual_history.py
    restarts Warp's loop at the checkpoints instead; trajectories are the
    same either way)."""
    points = sorted(set(int(i) for i in checkpoints if int(i) > 0))
    prev = getattr(_sampler, "active", None)
    _sampler.active = (points, observe)
    try:
        yield
    finally:
        _sampler.active = prev


def _report(points, observe, hist, nit, maxiter):
    observe(0, float(hist[0]))
    for stop in sorted(set([p for p in points if p <= maxiter] + [int(maxiter)])):
        if stop >= nit:
            observe(nit, float(hist[nit]))
            break
        observe(stop, float(hist[stop]))


def _cached_solver(method, A, M, use_cuda_graph) -> Solver:
    """One Solver per (operator, preconditioner, method, graph flag), kept on
    the operator, so repeated cg / cr calls replay the captured graph
    instead of capturing a new one (it is rebuilt only for new b / x)."""
    cache = A.__dict__.setdefault("_gbpc_solvers", [])
    for entry in cache:
        if entry[0] == method and entry[1] is M and entry[2] == bool(use_cuda_graph):
            return entry[3]
    s = Solver(method, A, M, use_cuda_graph)
    cache.append((method, M, bool(use_cuda_graph), s))
    if len(cache) > 4:
        cache.pop(0)
    return s


def _solve(method, A, b, x, tol, atol, maxiter, M, callback, check_every, use_cuda_graph):
    if callback is not None:
        raise NotImplementedError("per-iteration callbacks are not supported; the loop runs on "
                                  "the device")
    A = aslinearoperator(A)
    M = aslinearoperator(M)
    if b.dtype != x.dtype or b.shape != x.shape:
        raise TypeError("b and x must have the same dtype and shape")
    if b.dtype not in (torch.float32, torch.float64):
        raise TypeError("cg/cr run on float32 or float64 vectors")
    if A.dtype != b.dtype or (M is not None and M.dtype != b.dtype):
        raise TypeError("operator and vector dtypes differ")
    tol = 1.0e-5 if tol is None else float(tol)
    atol = 0.0 if atol is None else float(atol)
    native = (b.dtype == torch.float64 and getattr(A, "_op", None) is not None
              and (M is None or getattr(M, "_op", None) is not None))
    sampler = getattr(_sampler, "active", None)
    limit = int(maxiter) if int(maxiter) > 0 else b.numel()
    if not native:
        hist = [] if sampler else None
        it, rr, atol_sq = _host_krylov(method, A, M, b, x, tol, atol, int(maxiter), hist)
        if sampler:
            _report(sampler[0], sampler[1], hist, it, limit)
        if check_every == 0:
            dev = b.device
            return (torch.tensor([it], dtype=torch.int32, device=dev),
                    torch.tensor([rr], dtype=torch.float64, device=dev),
                    torch.tensor([atol_sq], dtype=torch.float64, device=dev))
        return it, math.sqrt(max(rr, 0.0)), math.sqrt(atol_sq)
    s = _cached_solver(method, A, M, use_cuda_graph)
    hist = torch.empty(limit + 1, dtype=torch.float64, device=b.device) if sampler else None
    nit, rr, atol_sq = s.run(b, x, tol, atol, maxiter, history=hist)
    if sampler:
        _report(sampler[0], sampler[1], hist.cpu().numpy(), int(nit.item()), limit)
    if check_every == 0:
        return nit.clone(), rr.clone(), atol_sq.clone()
    vals = torch.stack([nit.to(torch.float64), rr, atol_sq]).cpu()
    return int(vals[0]), math.sqrt(max(float(vals[1]), 0.0)), math.sqrt(float(vals[2]))


def cg(A, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10,
       use_cuda_graph=True):
    """Preconditioned conjugate gradient (warp.optim.linear.cg signature)."""
    return _solve("cg", A, b, x, tol, atol, maxiter, M, callback, check_every, use_cuda_graph)


def cr(A, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10,
       use_cuda_graph=True):
    """Preconditioned conjugate residual (warp.optim.linear.cr signature)."""
    return _solve("cr", A, b, x, tol, atol, maxiter, M, callback, check_every, use_cuda_graph)


class GmresSolver:
    """Reusable restarted GMRES bound to (A, M); repeated runs replay one graph."""

    def __init__(self, A, M=None, restart=31, use_cuda_graph=True):
        if isinstance(restart, bool) or not isinstance(restart, int) or not 1 <= restart <= 64:
            raise ValueError("restart must be an integer in [1, 64]")
        self.A = aslinearoperator(A)
        self.M = aslinearoperator(M)
        self.restart = restart
        self.use_graph = bool(use_cuda_graph)
        out = ctypes.c_void_p()
        _lib.call("gbpc_gmres_create", _handle(self.A), _handle(self.M), restart,
                  _lib.stream(self.A.device), ctypes.byref(out))
        self._h = out
        dev = self.A.device
        self.nit = torch.zeros(1, dtype=torch.int32, device=dev)
        self.res = torch.zeros(1, dtype=torch.float64, device=dev)
        self.target = torch.zeros(1, dtype=torch.float64, device=dev)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.load().gbpc_gmres_destroy(h)
            except Exception:
                pass

    @property
    def device_bytes(self) -> int:
        return _lib.object_bytes("gbpc_gmres_device_bytes", self._h)

    def run(self, b, x, tol=None, atol=None, maxiter=0):
        tol = 1.0e-5 if tol is None else float(tol)
        atol = 0.0 if atol is None else float(atol)
        _lib.call("gbpc_gmres_run", self._h, _lib.ptr(_flat(b)), _lib.ptr(_flat(x)), tol, atol,
                  int(maxiter), int(self.use_graph), _lib.ptr(self.nit), _lib.ptr(self.res),
                  _lib.ptr(self.target), _lib.stream(self.A.device))
        return self.nit, self.res, self.target


def gmres(A, b, x, tol=None, atol=None, restart=31, maxiter=0, M=None, callback=None,
          check_every=31, use_cuda_graph=True, is_left_preconditioner=False):
    """Restarted GMRES (warp.optim.linear.gmres signature), right-preconditioned.

    Returns (steps, residual norm, target) -- device arrays when
    ``check_every=0``, host numbers otherwise.  The residual norm is
    ``|b - A x|`` as tracked by the Givens recurrence; the loop stops when it
    is at most ``max(atol, tol |b|)`` or after ``maxiter`` Arnoldi steps.
    """
    if callback is not None:
        raise NotImplementedError("per-iteration callbacks are not supported; the loop runs on "
                                  "the device")
    if is_left_preconditioner:
        raise NotImplementedError("only right preconditioning is implemented")
    if b.dtype != torch.float64 or x.dtype != torch.float64:
        raise TypeError("gmres runs on float64 vectors")
    s = GmresSolver(A, M, restart, use_cuda_graph)
    nit, res, target = s.run(b, x, tol, atol, maxiter)
    if check_every == 0:
        return nit.clone(), res.clone(), target.clone()
    vals = torch.stack([nit.to(torch.float64), res, target]).cpu()
    return int(vals[0]), float(vals[1]), float(vals[2])
