"""Device GMRES against the oracle's textbook GMRES and the reference's
lifted-biharmonic test (tests/test_biharmonic.py:11-43)."""

import numpy as np
import pytest
import scipy.sparse as ss
import torch

from gpu_helpers import cuda, oracle_csr, to_bsr, vec

pytestmark = pytest.mark.gpu


def nonsymmetric(n, seed):
    rng = np.random.default_rng(seed)
    a = ss.random(n, n, density=0.06, random_state=rng) + ss.diags(4 + rng.uniform(0, 1, n))
    a = a.tocsr()
    a.sort_indices()
    return a, rng.normal(size=n)


@pytest.mark.parametrize("tau", [0.02, 2.0])
def test_lifted_equivalence(tau):
    from warp_preconditioners_gb300 import BiharmonicSystem, linear

    rng = np.random.default_rng(13)
    k = rng.normal(size=(10, 10))
    k = k @ k.T
    mass = rng.uniform(0.4, 2.0, size=10)
    b_np = rng.normal(size=10)
    system = BiharmonicSystem(to_bsr(k), vec(mass), tau)
    Q = np.diag(mass) + tau * (k / mass) @ k
    b = system.rhs(vec(b_np))
    x = torch.zeros_like(b)
    pre = system.preconditioner(max_row_size=10, kap_tolerance=0)
    h_inv = np.linalg.inv(np.diag(mass) + np.sqrt(tau) * k)
    v = vec(rng.normal(size=(10, 2)))
    out = torch.empty_like(v)
    pre.matvec(v, out, out, 1.0, 0.0)
    np.testing.assert_allclose(out.cpu().numpy(), h_inv @ v.cpu().numpy(), atol=1e-11)
    linear.gmres(system.matrix, b, x, M=pre, tol=1e-12, maxiter=100, restart=20)
    u = system.solution(x).cpu().numpy()
    np.testing.assert_allclose(u, np.linalg.solve(Q, b_np), rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(Q @ u, b_np, rtol=1e-9, atol=1e-9)
    actual = system.matrix.dense()
    expect = np.zeros((20, 20))
    expect[::2, ::2] = np.diag(mass)
    expect[1::2, 1::2] = np.diag(mass)
    expect[::2, 1::2] = -np.sqrt(tau) * k
    expect[1::2, ::2] = np.sqrt(tau) * k
    np.testing.assert_allclose(actual, expect)


@pytest.mark.parametrize("restart", [5, 30])
@pytest.mark.parametrize("precond", [False, True])
def test_gmres_matches_textbook_oracle(oracle, restart, precond):
    from warp_preconditioners_gb300 import linear

    a, b_np = nonsymmetric(300, 5)
    A = to_bsr(a)
    M = linear.preconditioner(A, "diag") if precond else None
    b = vec(b_np)
    x = torch.zeros_like(b)
    nit, res, tgt = linear.gmres(A, b, x, M=M, tol=1e-10, restart=restart, maxiter=500)
    om = oracle.Operator.diagonal(1 / a.diagonal()) if precond else None
    xo, ito, reso, tgto = oracle.gmres(oracle.Operator.csr(oracle_csr(oracle, a)), b_np, M=om,
                                       tol=1e-10, restart=restart, maxiter=500)
    assert abs(nit - ito) <= 1, (nit, ito)
    assert res <= tgt
    np.testing.assert_allclose(tgt, tgto, rtol=1e-14)
    np.testing.assert_allclose(x.cpu().numpy(), xo, rtol=1e-8, atol=1e-10)
    assert np.linalg.norm(b_np - a @ x.cpu().numpy()) <= 2 * tgt


def test_gmres_maxiter_device_returns_and_host_loop():
    from warp_preconditioners_gb300 import linear

    a, b_np = nonsymmetric(200, 6)
    A = to_bsr(a)
    b = vec(b_np)
    x = torch.zeros_like(b)
    nit, res, tgt = linear.gmres(A, b, x, tol=1e-14, restart=4, maxiter=7, check_every=0)
    assert isinstance(nit, torch.Tensor) and nit.is_cuda
    assert int(nit.item()) == 7 and float(res.item()) > float(tgt.item())
    # The host-driven loop runs the same kernels: identical iterates.
    x2 = torch.zeros_like(b)
    linear.gmres(A, b, x2, tol=1e-14, restart=4, maxiter=7, use_cuda_graph=False)
    assert torch.equal(x, x2)
    # A solver object replays its graph: same result again.
    s = linear.GmresSolver(A, None, restart=4)
    x3 = torch.zeros_like(b)
    s.run(b, x3, 1e-14, 0.0, 7)
    x3.zero_()
    s.run(b, x3, 1e-14, 0.0, 7)
    torch.cuda.synchronize()
    assert torch.equal(x, x3)
    with pytest.raises(NotImplementedError):
        linear.gmres(A, b, x, is_left_preconditioner=True)
    with pytest.raises(ValueError):
        linear.GmresSolver(A, None, restart=65)


def test_gmres_block_ilu_preconditioned_coupling(oracle):
    # Nonsymmetric 2x2-block system preconditioned by BlockILU0, as the
    # reference's indefinite tests do (tests/test_indefinite.py:127-139).
    from warp_preconditioners_gb300 import BlockILU0, linear

    rng = np.random.default_rng(61)
    n = 60
    lap = ss.diags([-1, 2.5, -1.2], [-1, 0, 1], shape=(n, n))
    c = np.array([[1.0, 0.3], [-0.4, 0.8]])
    a = ss.kron(lap, c).tocsr()
    a.sort_indices()
    A = to_bsr(a, block=2)
    truth = rng.normal(size=2 * n)
    b = vec(a @ truth)
    x = torch.zeros_like(b)
    nit, res, tgt = linear.gmres(A, b, x, M=BlockILU0(A, factor_sweeps=20, solve_sweeps=n),
                                 tol=1e-11, maxiter=60, restart=15)
    np.testing.assert_allclose(x.cpu().numpy(), truth, rtol=1e-8, atol=1e-8)
