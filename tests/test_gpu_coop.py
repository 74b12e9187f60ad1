"""Small systems solved by one kernel on one thread-block cluster (the
graph loop's replacement when a CG iteration needs at most ~600k
multiply-adds, for a scalar sparse or factored squared-Laplacian operator
with an FSAI or no preconditioner; larger systems, here the 40^3 ones, keep
the graph loop): the same method and stopping rule as the loop of separate
kernels (`use_cuda_graph=False` runs those), so iteration counts agree to
rounding and both reach the oracle's PCG; repeated runs give the same bits;
maxiter and a converged start behave like CG."""

import numpy as np
import pytest
import torch

from gpu_helpers import oracle_csr, to_bsr, vec

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["lap64", "lap3d40", "lap96_nopre"])
def test_coop_matches_kernel_loop_and_oracle(oracle, case):
    from warp_preconditioners_gb300 import FSAI, linear, problems

    if case == "lap64":
        a = problems.laplacian_2d(64)
    elif case == "lap3d40":
        a = problems.laplacian_3d(40)  # 64,000 rows: the largest size class
    else:
        a = problems.laplacian_2d(96)
    A = to_bsr(a)
    pre = None if case.endswith("nopre") else FSAI(A, max_row_size=8)
    b_np = problems.uniform_rhs(a.shape[0], 4)
    b = vec(b_np)
    coop = linear.Solver("cg", A, pre)
    loop = linear.Solver("cg", A, pre, use_cuda_graph=False)
    x1, x2 = torch.zeros_like(b), torch.zeros_like(b)
    n1, rr1, t1 = coop.run(b, x1, tol=1e-8, maxiter=5000)
    n2, rr2, t2 = loop.run(b, x2, tol=1e-8, maxiter=5000)
    n1, n2 = int(n1.item()), int(n2.item())
    assert rr1.item() <= t1.item() and rr2.item() <= t2.item()
    assert abs(n1 - n2) <= max(2, int(0.02 * n2)), (n1, n2)
    scale = np.abs(x2.cpu().numpy()).max()
    np.testing.assert_allclose(x1.cpu().numpy(), x2.cpu().numpy(), rtol=0, atol=1e-6 * scale)
    res = np.linalg.norm(b_np - a @ x1.cpu().numpy()) / np.linalg.norm(b_np)
    assert res <= 1.01e-8
    if pre is not None and case == "lap64":
        g, gt, _ = oracle.fsai(oracle_csr(oracle, a), width=8)
        _, it_or, _, _ = oracle.krylov("cg", oracle.Operator.csr(oracle_csr(oracle, a)), b_np,
                                       M=oracle.Operator.fsai(g, gt), tol=1e-8, maxiter=5000)
        assert abs(n1 - it_or) <= 2, (n1, it_or)
    x3 = torch.zeros_like(b)
    coop.run(b, x3, tol=1e-8, maxiter=5000)
    assert torch.equal(x1, x3)


def test_coop_maxiter_and_converged_start():
    from warp_preconditioners_gb300 import FSAI, linear, problems

    a = problems.laplacian_2d(48)
    A = to_bsr(a)
    b = vec(problems.uniform_rhs(a.shape[0], 5))
    s = linear.Solver("cg", A, FSAI(A))
    x = torch.zeros_like(b)
    nit, rr, atol_sq = s.run(b, x, tol=1e-14, maxiter=9)
    assert int(nit.item()) == 9 and rr.item() > atol_sq.item()
    x.zero_()
    s.run(b, x, tol=1e-10, maxiter=2000)
    nit, rr, atol_sq = s.run(b, x, tol=1e-6, maxiter=2000)
    assert int(nit.item()) == 0 and rr.item() <= atol_sq.item()


@pytest.mark.parametrize("side", [12, 40])
def test_coop_factored_operator_matches_kernel_loop_and_oracle(oracle, side):
    # The smoothing system's factored operator (every vertex free) with its
    # FSAI: 1,728 rows run on one cluster, 64,000 on a cooperative grid.
    from warp_preconditioners_gb300 import FSAI, SquaredLaplacianOperator, from_scipy, linear, problems

    verts, tets, K, mass = problems.tet_cube(side)
    Q = problems.biharmonic(K, mass, 1e-4)
    n = Q.shape[0]
    dev = torch.device("cuda:0")
    op = SquaredLaplacianOperator(from_scipy(K, dev), vec(mass),
                                  torch.arange(n, dtype=torch.int32, device=dev), mass_weight=1e-4)
    pre = FSAI(from_scipy(Q, dev), max_row_size=8)
    b_np = problems.smoothing_rhs(verts, mass, 1e-4)[0]
    b = vec(b_np)
    x1, x2 = torch.zeros_like(b), torch.zeros_like(b)
    n1, rr1, t1 = linear.Solver("cg", op, pre).run(b, x1, tol=1e-8, maxiter=20000)
    n2, _, _ = linear.Solver("cg", op, pre, use_cuda_graph=False).run(b, x2, tol=1e-8,
                                                                     maxiter=20000)
    n1, n2 = int(n1.item()), int(n2.item())
    assert rr1.item() <= t1.item()
    assert abs(n1 - n2) <= max(2, int(0.02 * n2)), (n1, n2)

    def berr(x):
        return float(np.max(np.abs(b_np - Q @ x) / (abs(Q) @ np.abs(x) + np.abs(b_np))))

    assert berr(x1.cpu().numpy()) <= max(4 * berr(x2.cpu().numpy()), 1e-14)
    if side == 12:
        qc = oracle.CSR(Q.indptr, Q.indices, Q.data)
        g, gt, _ = oracle.fsai(qc, width=8)
        kc = oracle.CSR(K.indptr, K.indices, K.data)
        _, it_or, _, _ = oracle.krylov("cg", oracle.Operator.sqlap(kc, mass, 1e-4), b_np,
                                       M=oracle.Operator.fsai(g, gt), tol=1e-8, maxiter=20000)
        assert abs(n1 - it_or) <= max(2, int(0.02 * it_or)), (n1, it_or)
