"""Residual sampling (linear.sample_iterations) leaves the CG / CR
trajectories unchanged: the reference's check of its diagnostic sampler
(tests/test_residual_history.py:16-31: a diagonal 30 x 30 system with
eigenvalues 1..1e4, 37 iterations, checkpoints 1, 2, 7, 19, 37) on the
device-resident loop and on the host-stepped loop of a Python operator."""

import numpy as np
import pytest
import torch

from gpu_helpers import to_bsr, vec

pytestmark = pytest.mark.gpu


def _system():
    a = np.diag(np.geomspace(1.0, 1e4, 30))
    b = np.random.default_rng(3).normal(size=30)
    return a, b


@pytest.mark.parametrize("method", ["cg", "cr"])
@pytest.mark.parametrize("python_operator", [False, True])
def test_sampling_preserves_recurrence(method, python_operator):
    from warp_preconditioners_gb300 import SparseOperator, linear
    from warp_preconditioners_gb300.linear import LinearOperator

    a, b_np = _system()
    A = SparseOperator(to_bsr(a))
    if python_operator:
        inner = A
        A = LinearOperator(inner.shape, inner.dtype, inner.device,
                           lambda x, y, z, al, be: inner.matvec(x, y, z, al, be))
    solve = linear.cg if method == "cg" else linear.cr
    b = vec(b_np)
    native, sampled = torch.zeros_like(b), torch.zeros_like(b)
    n0, r0, _ = solve(A, b, native, tol=0.0, atol=0.0, maxiter=37, check_every=0)
    obs = []
    with linear.sample_iterations([1, 2, 7, 19, 37], lambda i, r: obs.append((i, r))):
        nit, rnorm, _ = solve(A, b, sampled, tol=0.0, atol=0.0, maxiter=37, check_every=0)
    assert int(nit.item()) == 37
    assert [i for i, _ in obs] == [0, 1, 2, 7, 19, 37]
    assert torch.equal(native, sampled)
    assert obs[0][1] == pytest.approx(np.linalg.norm(b_np), rel=1e-14)
    assert obs[-1][1] == pytest.approx(float(np.sqrt(rnorm.item())), rel=1e-14)
    # an early stop is observed where it happens
    obs.clear()
    with linear.sample_iterations([5, 500], lambda i, r: obs.append((i, r))):
        nit2, _, _ = solve(A, b, torch.zeros_like(b), tol=1e-6, maxiter=1000, check_every=0)
    assert [i for i, _ in obs] == [0, 5, int(nit2.item())]
    assert 5 < int(nit2.item()) < 500
