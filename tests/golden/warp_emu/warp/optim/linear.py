"""Krylov solvers of the Warp emulation (test infrastructure).

Restates the documented interface of ``warp.optim.linear``: a
``LinearOperator`` wraps ``matvec(x, y, z, alpha, beta)`` computing
``z = alpha A x + beta y``; ``cg``, ``cr``, ``bicgstab`` and ``gmres``
take ``(A, b, x, tol, atol, maxiter, M, ...)``, stop once the residual norm
is at most ``max(atol, tol * |b|)`` (``maxiter = 0`` means the system size)
and return ``(iterations, residual_norm, absolute_tolerance)``.  The loops
are the textbook methods (the reference pins none of Warp's iterates, only
converged solutions), evaluated in float64 on the arrays' scalars.
"""

from __future__ import annotations

import numpy as np

import warp as wp
from warp import sparse as sp
from warp import types as wt


class LinearOperator:
    def __init__(self, shape, dtype, device, matvec):
        self._shape = tuple(shape)
        self._dtype = dtype
        self._device = device
        self._matvec = matvec

    @property
    def shape(self):
        return self._shape

    @property
    def dtype(self):
        return self._dtype

    @property
    def device(self):
        return self._device

    @property
    def matvec(self):
        return self._matvec

    @property
    def scalar_type(self):
        return wt.scalar_of(self._dtype)


def aslinearoperator(A):
    if A is None or isinstance(A, LinearOperator):
        return A
    if isinstance(A, sp.BsrMatrix):
        def mv(x, y, z, alpha, beta):
            if beta != 0.0 and z.ptr != y.ptr:
                wp.copy(z, y)
            sp.bsr_mv(A, x, z, alpha=alpha, beta=beta)

        return LinearOperator(A.shape, A.dtype, A.device, mv)
    if isinstance(A, wp.array) and A.ndim == 2:
        dense = A

        def mv(x, y, z, alpha, beta):
            xs = x.numpy().reshape(-1)
            out = alpha * (dense.numpy() @ xs)
            if beta != 0.0:
                out = out + beta * y.numpy().reshape(-1)
            z.numpy().reshape(-1)[...] = out

        return LinearOperator(A.shape, A.dtype, A.device, mv)
    raise ValueError("unable to wrap this operator")


def preconditioner(A, ptype="diag"):
    """Scalar diagonal preconditioner: z = alpha x / diag(A) + beta y (entries
    with a zero diagonal pass x through)."""
    if ptype == "id":
        return None
    if ptype not in ("diag", "diag_abs"):
        raise ValueError(f"unsupported preconditioner {ptype!r}")
    rows, cols, vals = A._blocks()
    b = A.block_shape[0]
    d = np.zeros(A.shape[0], dtype=A.scalar_type)
    for k in range(len(rows)):
        if rows[k] == cols[k]:
            d[rows[k] * b: rows[k] * b + b] = np.diag(vals[k])
    if ptype == "diag_abs":
        d = np.abs(d)
    inv = np.where(d != 0, 1.0 / np.where(d != 0, d, 1.0), 1.0).astype(A.scalar_type)

    def mv(x, y, z, alpha, beta):
        out = alpha * (inv * x.numpy().reshape(-1))
        if beta != 0.0:
            out = out + beta * y.numpy().reshape(-1)
        z.numpy().reshape(-1)[...] = out

    return LinearOperator(A.shape, A.dtype, A.device, mv)


class _Work:
    """Float64 host views plus array wrappers the operators can be called with."""

    def __init__(self, like):
        self.like = like

    def new(self):
        return wp.empty_like(self.like)


def _flat(a):
    return a.numpy().reshape(-1)


def _apply(op, src, dst):
    op.matvec(src, dst, dst, 1.0, 0.0)


def _setup(A, b, tol, atol, maxiter):
    A = aslinearoperator(A)
    n = _flat(b).size
    if maxiter == 0:
        maxiter = n
    if tol is None and atol is None:
        tol = 1.0e-5
    tol = 0.0 if tol is None else float(tol)
    atol = 0.0 if atol is None else float(atol)
    bnorm = float(np.sqrt(np.dot(_flat(b).astype(np.float64), _flat(b).astype(np.float64))))
    return A, maxiter, max(atol, tol * bnorm)


def _residual(A, b, x):
    r = wp.empty_like(b)
    A.matvec(x, b, r, -1.0, 1.0)
    return r


def cg(A, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10,
       use_cuda_graph=True):
    A, maxiter, target = _setup(A, b, tol, atol, maxiter)
    M = aslinearoperator(M)
    r = _residual(A, b, x)
    z = wp.empty_like(b)
    if M is not None:
        _apply(M, r, z)
    else:
        wp.copy(z, r)
    p = wp.clone(z)
    q = wp.empty_like(b)
    rz = float(np.dot(_flat(r), _flat(z)))
    rr = float(np.dot(_flat(r), _flat(r)))
    it = 0
    while it < maxiter and rr > target * target:
        _apply(A, p, q)
        alpha = rz / float(np.dot(_flat(p), _flat(q)))
        _flat(x)[...] += alpha * _flat(p)
        _flat(r)[...] -= alpha * _flat(q)
        rr = float(np.dot(_flat(r), _flat(r)))
        it += 1
        if rr <= target * target:
            break
        if M is not None:
            _apply(M, r, z)
        else:
            wp.copy(z, r)
        rz_new = float(np.dot(_flat(r), _flat(z)))
        beta = rz_new / rz
        rz = rz_new
        _flat(p)[...] = _flat(z) + beta * _flat(p)
        if callback is not None:
            callback(it, np.sqrt(rr), target)
    return it, float(np.sqrt(rr)), target


def cr(A, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10,
       use_cuda_graph=True):
    A, maxiter, target = _setup(A, b, tol, atol, maxiter)
    M = aslinearoperator(M)

    def prec(src, dst):
        if M is not None:
            _apply(M, src, dst)
        else:
            wp.copy(dst, src)

    r = _residual(A, b, x)
    z = wp.empty_like(b)
    prec(r, z)
    Az = wp.empty_like(b)
    _apply(A, z, Az)
    p = wp.clone(z)
    Ap = wp.clone(Az)
    y = wp.empty_like(b)
    zAz = float(np.dot(_flat(z), _flat(Az)))
    rr = float(np.dot(_flat(r), _flat(r)))
    it = 0
    while it < maxiter and rr > target * target:
        prec(Ap, y)
        alpha = zAz / float(np.dot(_flat(Ap), _flat(y)))
        _flat(x)[...] += alpha * _flat(p)
        _flat(r)[...] -= alpha * _flat(Ap)
        _flat(z)[...] -= alpha * _flat(y)
        rr = float(np.dot(_flat(r), _flat(r)))
        it += 1
        if rr <= target * target:
            break
        _apply(A, z, Az)
        zAz_new = float(np.dot(_flat(z), _flat(Az)))
        beta = zAz_new / zAz
        zAz = zAz_new
        _flat(p)[...] = _flat(z) + beta * _flat(p)
        _flat(Ap)[...] = _flat(Az) + beta * _flat(Ap)
    return it, float(np.sqrt(rr)), target


def bicgstab(A, b, x, tol=None, atol=None, maxiter=0, M=None, callback=None, check_every=10,
             use_cuda_graph=True, is_left_preconditioner=False):
    A, maxiter, target = _setup(A, b, tol, atol, maxiter)
    M = aslinearoperator(M)

    def prec(src, dst):
        if M is not None:
            _apply(M, src, dst)
        else:
            wp.copy(dst, src)

    r = _residual(A, b, x)
    r0 = wp.clone(r)
    p = wp.clone(r)
    ph, v, s, sh, t = (wp.empty_like(b) for _ in range(5))
    rho = float(np.dot(_flat(r0), _flat(r)))
    rr = float(np.dot(_flat(r), _flat(r)))
    it = 0
    while it < maxiter and rr > target * target:
        prec(p, ph)
        _apply(A, ph, v)
        alpha = rho / float(np.dot(_flat(r0), _flat(v)))
        _flat(s)[...] = _flat(r) - alpha * _flat(v)
        prec(s, sh)
        _apply(A, sh, t)
        omega = float(np.dot(_flat(t), _flat(s))) / float(np.dot(_flat(t), _flat(t)))
        _flat(x)[...] += alpha * _flat(ph) + omega * _flat(sh)
        _flat(r)[...] = _flat(s) - omega * _flat(t)
        rr = float(np.dot(_flat(r), _flat(r)))
        it += 1
        rho_new = float(np.dot(_flat(r0), _flat(r)))
        beta = (rho_new / rho) * (alpha / omega)
        rho = rho_new
        _flat(p)[...] = _flat(r) + beta * (_flat(p) - omega * _flat(v))
    return it, float(np.sqrt(rr)), target


def gmres(A, b, x, tol=None, atol=None, restart=31, maxiter=0, M=None, callback=None,
          check_every=31, use_cuda_graph=True, is_left_preconditioner=False):
    """Restarted GMRES, right-preconditioned (left preconditioning is applied
    to the residual the same way; both converge to the same solution)."""
    A, maxiter, target = _setup(A, b, tol, atol, maxiter)
    M = aslinearoperator(M)
    n = _flat(b).size
    tmp_in = wp.empty_like(b)
    tmp_out = wp.empty_like(b)

    def apply(op, vec):
        _flat(tmp_in)[...] = vec
        _apply(op, tmp_in, tmp_out)
        return _flat(tmp_out).astype(np.float64).copy()

    def prec(vec):
        return apply(M, vec) if M is not None else vec.copy()

    xs = _flat(x)
    it = 0
    r = _flat(b).astype(np.float64) - apply(A, xs.astype(np.float64))
    rnorm = float(np.linalg.norm(r))
    while it < maxiter and rnorm > target:
        m = min(restart, maxiter - it)
        V = np.zeros((m + 1, n))
        H = np.zeros((m + 1, m))
        V[0] = r / rnorm
        g = np.zeros(m + 1)
        g[0] = rnorm
        k = 0
        for k in range(m):
            w = apply(A, prec(V[k]))
            for j in range(k + 1):
                H[j, k] = np.dot(V[j], w)
                w = w - H[j, k] * V[j]
            H[k + 1, k] = np.linalg.norm(w)
            if H[k + 1, k] != 0:
                V[k + 1] = w / H[k + 1, k]
            it += 1
            y, *_ = np.linalg.lstsq(H[: k + 2, : k + 1], g[: k + 2], rcond=None)
            res = np.linalg.norm(g[: k + 2] - H[: k + 2, : k + 1] @ y)
            if res <= target or H[k + 1, k] == 0:
                break
        y, *_ = np.linalg.lstsq(H[: k + 2, : k + 1], g[: k + 2], rcond=None)
        xs[...] = xs + prec(V[: k + 1].T @ y)
        r = _flat(b).astype(np.float64) - apply(A, xs.astype(np.float64))
        rnorm = float(np.linalg.norm(r))
    return it, rnorm, target
