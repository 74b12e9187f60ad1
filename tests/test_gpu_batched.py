"""Batched operators, batched PCG and mixed-precision refinement against the
single-vector GPU path and the assembled float64 operator."""

import numpy as np
import pytest
import torch

from gpu_helpers import cuda, to_bsr, vec

pytestmark = pytest.mark.gpu


def _block(rng, n, k, dtype=torch.float64):
    return torch.as_tensor(rng.normal(size=(n, k)), dtype=dtype, device=cuda()).contiguous()


@pytest.mark.parametrize("k", [1, 5, 32])
def test_batched_sparse_and_fsai_match_single_vector(k):
    from warp_preconditioners_gb300 import FSAI, SparseOperator, batched, problems

    a = problems.laplacian_2d(24)
    A = to_bsr(a)
    n = a.shape[0]
    rng = np.random.default_rng(k)
    X = _block(rng, n, k)
    Y = _block(rng, n, k)
    Z = torch.empty_like(X)
    batched.batched_sparse(A).apply(X, Y, Z, 0.7, -0.3)
    single = SparseOperator(A)
    pre = FSAI(A, max_row_size=8)
    bf = batched.batched_fsai(pre)
    Zf = torch.empty_like(X)
    bf.apply(X, Y, Zf, 1.3, 0.2)
    for j in range(k):
        x, y = X[:, j].contiguous(), Y[:, j].contiguous()
        z = torch.empty_like(x)
        single.matvec(x, y, z, 0.7, -0.3)
        torch.testing.assert_close(Z[:, j], z, rtol=1e-12, atol=1e-12)
        pre.matvec(x, y, z, 1.3, 0.2)
        torch.testing.assert_close(Zf[:, j], z, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("factor_dtype,tol", [(torch.float32, 2e-5), (torch.bfloat16, 2e-2)])
def test_batched_low_precision_fsai(factor_dtype, tol):
    from warp_preconditioners_gb300 import FSAI, batched, problems

    a = problems.laplacian_2d(24)
    pre = FSAI(to_bsr(a), max_row_size=8)
    g = pre.G.dense()
    n, k = a.shape[0], 8
    X64 = _block(np.random.default_rng(3), n, k)
    X = X64.to(torch.float32).contiguous()
    Z = torch.empty_like(X)
    batched.batched_fsai(pre, factor_dtype, torch.float32).apply(X, None, Z, 1.0, 0.0)
    ref = g.T @ (g @ X64.cpu().numpy())
    err = np.abs(Z.cpu().double().numpy() - ref).max() / np.abs(ref).max()
    assert err < tol


def test_batched_sqlap_matches_single_vector():
    from warp_preconditioners_gb300 import SquaredLaplacianOperator, batched, problems

    _, _, K, mass = problems.tet_cube(8)
    n, k = K.shape[0], 6
    L = to_bsr(K)
    m = vec(mass)
    op = SquaredLaplacianOperator(L, m, torch.arange(n, dtype=torch.int32, device=cuda()),
                                  mass_weight=1e-4)
    bop = batched.batched_sqlap(L, m, 1e-4)
    X = _block(np.random.default_rng(5), n, k)
    Z = torch.empty_like(X)
    bop.apply(X, X, Z, 0.5, 0.25)
    for j in range(k):
        x = X[:, j].contiguous()
        z = torch.empty_like(x)
        op.matvec(x, x, z, 0.5, 0.25)
        torch.testing.assert_close(Z[:, j], z, rtol=1e-11, atol=1e-14)


def test_batched_cg_matches_single_solves():
    from warp_preconditioners_gb300 import FSAI, batched, linear, problems

    a = problems.laplacian_2d(40)
    A = to_bsr(a)
    pre = FSAI(A, max_row_size=8)
    n, k = a.shape[0], 7
    B = torch.as_tensor(np.stack([problems.uniform_rhs(n, s) for s in range(k)], 1),
                        device=cuda()).contiguous()
    X = torch.zeros_like(B)
    solver = batched.BatchedCG(batched.batched_sparse(A), batched.batched_fsai(pre))
    nit, rr = solver.run(B, X, tol=1e-10, maxiter=2000)
    nit = nit.cpu().numpy()
    for j in range(k):
        x = torch.zeros(n, dtype=torch.float64, device=cuda())
        it, res, atol = linear.cg(A, B[:, j].contiguous(), x, tol=1e-10, maxiter=2000, M=pre)
        assert abs(int(nit[j]) - it) <= 2
        np.testing.assert_allclose(X[:, j].cpu().numpy(), x.cpu().numpy(), rtol=1e-7,
                                   atol=1e-9 * np.abs(x.cpu().numpy()).max())
        assert np.linalg.norm(B[:, j].cpu().numpy() - a @ X[:, j].cpu().numpy()) <= \
            1.01e-10 * np.linalg.norm(B[:, j].cpu().numpy())


@pytest.mark.parametrize("factor_dtype", [torch.float32, torch.bfloat16])
def test_mixed_precision_refinement_reaches_float64_backward_error(factor_dtype):
    from warp_preconditioners_gb300 import FSAI, batched, problems

    verts, _, K, mass = problems.tet_cube(14)
    alpha = 1e-4
    q = problems.biharmonic(K, mass, alpha)
    n, k = K.shape[0], 8
    pre = FSAI(to_bsr(q), max_row_size=8)
    solver = batched.MixedPrecisionSolver(to_bsr(K), vec(mass), alpha, pre, factor_dtype)
    b_np = np.stack([problems.uniform_rhs(n, s) for s in range(k)], 1)
    B = torch.as_tensor(b_np, device=cuda()).contiguous()
    X = torch.zeros_like(B)
    outer, inner = solver.solve(B, X, tol_outer=1e-12, tol_inner=1e-3, max_outer=30)
    x = X.cpu().numpy()
    absq = abs(q)
    for j in range(k):
        berr = np.max(np.abs(b_np[:, j] - q @ x[:, j]) / (absq @ np.abs(x[:, j]) + np.abs(b_np[:, j])))
        assert berr <= 1e-10, (j, berr, outer[j], inner[j])
    assert max(outer) < 30
