"""Mixed harmonic systems and their preconditioners on the GPU, ported from
the reference's tests/test_indefinite.py:55-139 and :195-232 (numpy known
answers: block signs, Schur complement, MatchingSchur / ShiftedBlock applies,
GMRES solves, equilibration)."""

import numpy as np
import pytest
import torch

from gpu_helpers import cuda, to_bsr, vec

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order", [2, 3])
def test_mixed_signs_matching_and_gmres(order):
    from warp_preconditioners_gb300 import (BlockILU0, MatchingSchur, MixedHarmonicSystem,
                                            ShiftedBlock, linear)

    rng = np.random.default_rng(7)
    n = 7
    edges = rng.uniform(0.1, 0.3, size=(n, n))
    edges = (edges + edges.T) / 2
    k = np.diag(edges.sum(axis=1)) - edges
    mass = rng.uniform(0.7, 1.2, size=n)
    alpha = 0.04
    system = MixedHarmonicSystem(to_bsr(k), vec(mass), order=order, data_weight=alpha)
    M = np.diag(mass)
    zero = np.zeros_like(M)
    expected = (np.block([[alpha * M, -k], [-k, -M]]) if order == 2
                else np.block([[alpha * M, zero, -k], [zero, -k, -M], [-k, -M, zero]]))
    permutation = np.arange(n * order).reshape(order, n).T.ravel()
    expected = expected[np.ix_(permutation, permutation)]
    np.testing.assert_allclose(system.matrix.dense(), expected)
    primary = np.arange(0, n * order, order)
    auxiliary = np.setdiff1d(np.arange(n * order), primary)
    schur = expected[np.ix_(primary, primary)] - expected[np.ix_(primary, auxiliary)] @ \
        np.linalg.solve(expected[np.ix_(auxiliary, auxiliary)], expected[np.ix_(auxiliary, primary)])
    invmass = np.diag(1 / mass)
    target_schur = (alpha * M + k @ invmass @ k if order == 2
                    else alpha * M - k @ invmass @ k @ invmass @ k)
    np.testing.assert_allclose(schur, target_schur, rtol=1e-12, atol=1e-12)
    pre = MatchingSchur(system, max_row_size=n, kap_tolerance=0)
    x = vec(rng.normal(size=(n, order)))
    y = torch.empty_like(x)
    pre.matvec(x, y, y, 1.0, 0.0)
    r = x.cpu().numpy()
    H = k + alpha ** (1 / order) * M
    invH = np.linalg.inv(H)
    if order == 2:
        g = r[:, 0] - k @ (r[:, 1] / mass)
        u = invH @ M @ invH @ g
        result = np.column_stack([u, -(k @ u + r[:, 1]) / mass])
    else:
        g = r[:, 0] - k @ (r[:, 1] / mass) + k @ ((k @ (r[:, 2] / mass)) / mass)
        u = -invH @ M @ invH @ M @ invH @ g
        aux = -(k @ u + r[:, 2]) / mass
        result = np.column_stack([u, aux, -(k @ aux + r[:, 1]) / mass])
    np.testing.assert_allclose(y.cpu().numpy(), result, rtol=2e-11, atol=2e-11)
    shifted = ShiftedBlock(system, max_row_size=n, kap_tolerance=0)
    shifted.matvec(x, y, y, 1.0, 0.0)
    if order == 2:
        scale = alpha ** 0.25
        target = np.column_stack([
            invH @ ((r[:, 0] / scale - scale * r[:, 1]) * 0.5) / scale,
            invH @ ((-r[:, 0] / scale - scale * r[:, 1]) * 0.5) * scale,
        ])
    else:
        target = np.column_stack([-invH @ r[:, 2], -invH @ r[:, 1], -invH @ r[:, 0]])
    np.testing.assert_allclose(y.cpu().numpy(), target, rtol=1e-11, atol=1e-11)
    # Capturable: a graph replay gives the same result.
    y2 = torch.zeros_like(y)
    graph = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(graph, stream=s):
            shifted.matvec(x, y2, y2, 1.0, 0.0)
    torch.cuda.current_stream().wait_stream(s)
    graph.replay()
    torch.cuda.synchronize()
    np.testing.assert_allclose(y2.cpu().numpy(), target, rtol=1e-11, atol=1e-11)
    truth = rng.normal(size=(n, order))
    b = vec((expected @ truth.ravel()).reshape(n, order))
    solution = torch.zeros_like(b)
    linear.gmres(system.matrix, b, solution,
                 M=BlockILU0(system.matrix, factor_sweeps=20, solve_sweeps=n),
                 tol=1e-11, maxiter=60, restart=15)
    np.testing.assert_allclose(solution.cpu().numpy(), truth, rtol=1e-8, atol=1e-8)
    # The Schur preconditioner under GMRES as well.
    solution.zero_()
    linear.gmres(system.matrix, b, solution, M=pre, tol=1e-11, maxiter=200, restart=30)
    np.testing.assert_allclose(solution.cpu().numpy(), truth, rtol=1e-7, atol=1e-7)


@pytest.mark.parametrize("order", [2, 3])
def test_mixed_equilibration_preserves_equations(order):
    from warp_preconditioners_gb300 import MixedHarmonicSystem, ShiftedBlock, linear

    n = 5
    k = np.diag(np.full(n, 2.0)) - np.diag(np.ones(n - 1), 1) - np.diag(np.ones(n - 1), -1)
    mass = np.linspace(0.6, 1.3, n)
    K = to_bsr(k)
    mw = vec(mass)
    original = MixedHarmonicSystem(K, mw, order=order, data_weight=1e-4)
    balanced = MixedHarmonicSystem(K, mw, order=order, data_weight=1e-4, equilibrate=True)
    a = original.matrix.dense()
    s = np.tile(np.asarray(balanced.scale), n)
    np.testing.assert_allclose(balanced.matrix.dense(), s[:, None] * a * s[None, :], rtol=1e-12,
                               atol=1e-12)
    b = vec(np.linspace(-1, 1, n))
    rhs = balanced.rhs(b)
    np.testing.assert_allclose(rhs.cpu().numpy().ravel(), original.rhs(b).cpu().numpy().ravel() * s)
    x = torch.zeros_like(rhs)
    linear.gmres(balanced.matrix, rhs, x, M=ShiftedBlock(balanced, max_row_size=n, kap_tolerance=0),
                 tol=1e-12, restart=15, maxiter=60)
    result = balanced.transform(x).cpu().numpy().ravel()
    np.testing.assert_allclose(a @ result, original.rhs(b).cpu().numpy().ravel(), atol=1e-9)
    np.testing.assert_array_equal(balanced.solution(x).cpu().numpy(),
                                  result.reshape(n, order)[:, 0])


def test_mixed_argument_checks():
    from warp_preconditioners_gb300 import MatchingSchur, MixedHarmonicSystem

    K = to_bsr(np.eye(3) * 2)
    with pytest.raises(ValueError, match="order"):
        MixedHarmonicSystem(K, vec(np.ones(3)), order=4)
    with pytest.raises(ValueError, match="finite positive"):
        MixedHarmonicSystem(K, vec([1.0, -1.0, 1.0]))
    s = MixedHarmonicSystem(K, vec(np.ones(3)))
    with pytest.raises(ValueError, match="must match H"):
        MatchingSchur(s, H_inverse=MixedHarmonicSystem(to_bsr(np.eye(4)), vec(np.ones(4))).H)
