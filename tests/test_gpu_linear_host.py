"""cg / cr beyond the device-resident float64 loop: operators written in
Python (no libgbpc handle), float32 systems, vec3d-shaped vectors, and the
solver cache of repeated calls.

warp.optim.linear's cg / cr accept any LinearOperator and any vector dtype
(the reference builds operators with ``super().__init__(shape, dtype,
device, matvec)``, warp_preconditioners/fsai.py:339, and runs float32
systems, tests/test_sparse_operator.py:13-24).  Here such calls run the
host-stepped loop over libgbpc's vector kernels; the float64 results are
checked against the oracle's textbook PCG / PCR and the device loop.
"""

import numpy as np
import pytest
import scipy.sparse as ss
import torch

from gpu_helpers import cuda, oracle_csr, to_bsr, vec

pytestmark = pytest.mark.gpu


def _python_operator(inner):
    """A LinearOperator whose matvec is Python code around another operator."""
    from warp_preconditioners_gb300.linear import LinearOperator

    def matvec(x, y, z, alpha, beta):
        inner.matvec(x, y, z, alpha, beta)

    return LinearOperator(inner.shape, inner.dtype, inner.device, matvec)


@pytest.mark.parametrize("method", ["cg", "cr"])
def test_python_operators_match_oracle_and_device_loop(oracle, method):
    from warp_preconditioners_gb300 import FSAI, SparseOperator, linear, problems

    a = problems.laplacian_2d(40)
    A = to_bsr(a)
    pre = FSAI(A, max_row_size=8)
    b_np = problems.uniform_rhs(a.shape[0], 3)
    b = vec(b_np)
    op, mp = _python_operator(SparseOperator(A)), _python_operator(pre)
    assert getattr(op, "_op", None) is None
    x = torch.zeros_like(b)
    it, res, tgt = linear.cg(op, b, x, tol=1e-8, maxiter=2000, M=mp) if method == "cg" else \
        linear.cr(op, b, x, tol=1e-8, maxiter=2000, M=mp)
    assert res <= tgt
    g, gt, _ = oracle.fsai(oracle_csr(oracle, a), width=8)
    x_or, it_or, _, _ = oracle.krylov(method, oracle.Operator.csr(oracle_csr(oracle, a)), b_np,
                                      M=oracle.Operator.fsai(g, gt), tol=1e-8, maxiter=2000)
    assert abs(it - it_or) <= 2, (it, it_or)
    np.testing.assert_allclose(x.cpu().numpy(), x_or, rtol=1e-6,
                               atol=1e-6 * np.abs(x_or).max())
    # The device loop on the native operators reaches the same solution.
    x2 = torch.zeros_like(b)
    solve = linear.cg if method == "cg" else linear.cr
    it2, _, _ = solve(A, b, x2, tol=1e-8, maxiter=2000, M=pre)
    assert abs(it - it2) <= 2
    np.testing.assert_allclose(x.cpu().numpy(), x2.cpu().numpy(), rtol=1e-6,
                               atol=1e-6 * np.abs(x_or).max())
    # device return values with check_every=0
    x.zero_()
    outs = linear.cg(op, b, x, tol=1e-8, maxiter=2000, M=mp, check_every=0)
    assert all(isinstance(t, torch.Tensor) and t.is_cuda for t in outs)


@pytest.mark.parametrize("method", ["cg", "cr"])
def test_float32_system(method):
    # A float32 operator and float32 FSAI (tests/test_fsai.py parametrises
    # both dtypes); the float32 solve agrees with the float64 one to float32
    # accuracy.
    from warp_preconditioners_gb300 import FSAI, linear, problems

    a = problems.laplacian_2d(32)
    b_np = problems.uniform_rhs(a.shape[0], 1)
    A32 = to_bsr(a, torch.float32)
    pre32 = FSAI(A32, max_row_size=8)
    b32 = vec(b_np, torch.float32)
    x32 = torch.zeros_like(b32)
    solve = linear.cg if method == "cg" else linear.cr
    it, res, tgt = solve(A32, b32, x32, tol=1e-5, maxiter=1000, M=pre32)
    assert res <= tgt and it > 0
    assert x32.dtype == torch.float32
    A64 = to_bsr(a)
    x64 = torch.zeros(a.shape[0], dtype=torch.float64, device=cuda())
    solve(A64, vec(b_np), x64, tol=1e-10, maxiter=1000, M=FSAI(A64, max_row_size=8))
    ref = x64.cpu().numpy()
    np.testing.assert_allclose(x32.cpu().double().numpy(), ref, rtol=1e-3,
                               atol=1e-3 * np.abs(ref).max())
    with pytest.raises(TypeError):
        solve(A32, vec(b_np), torch.zeros(a.shape[0], dtype=torch.float64, device=cuda()))


def test_vec3d_vectors_on_blocked_operator():
    # tests/test_sparse_operator.py:50-61: a 3x3-blocked operator and FSAI,
    # x and b shaped (23, 3) like wp.vec3d arrays.
    from warp_preconditioners_gb300 import FSAI, SparseOperator, linear

    n = 69
    a = ss.diags([-np.ones(n - 1), np.full(n, 2.1), -np.ones(n - 1)], [-1, 0, 1]).tocsr()
    raw = to_bsr(a, block=3)
    operator = SparseOperator(raw, row_lanes=8)
    pre = FSAI(raw, max_row_size=8, apply_lanes=4)
    x = torch.zeros((23, 3), dtype=torch.float64, device=cuda())
    b = torch.ones_like(x)
    linear.cg(operator, b, x, M=pre, tol=1e-12, maxiter=1000)
    np.testing.assert_allclose(a @ x.cpu().numpy().ravel(), 1.0, atol=1e-10)
    # the same through a Python operator (host-stepped loop)
    x.zero_()
    linear.cg(_python_operator(operator), b, x, M=_python_operator(pre), tol=1e-12,
              maxiter=1000)
    np.testing.assert_allclose(a @ x.cpu().numpy().ravel(), 1.0, atol=1e-10)


def test_repeated_calls_reuse_one_solver():
    from warp_preconditioners_gb300 import FSAI, linear, problems

    a = problems.laplacian_2d(24)
    A = to_bsr(a)
    pre = FSAI(A)
    b = vec(problems.uniform_rhs(a.shape[0], 2))
    xs = []
    for _ in range(3):
        x = torch.zeros_like(b)
        linear.cg(A, b, x, tol=1e-8, M=pre)
        xs.append(x)
    op = linear.aslinearoperator(A)
    solvers = [e[3] for e in op._gbpc_solvers]
    assert len(solvers) == 1
    assert torch.equal(xs[0], xs[1]) and torch.equal(xs[1], xs[2])
    linear.cr(A, b, torch.zeros_like(b), tol=1e-8, M=pre)
    assert len(op._gbpc_solvers) == 2
