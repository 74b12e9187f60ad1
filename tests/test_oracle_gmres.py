"""Oracle GMRES (textbook restarted, right-preconditioned) against direct
solves: the reference's GMRES call sites check the solution of the solved
system (tests/test_biharmonic.py:32-35, tests/test_indefinite.py:130-139)."""

import numpy as np
import scipy.sparse as ss

from oracle import oracle as O


def nonsymmetric(n, seed):
    rng = np.random.default_rng(seed)
    a = ss.random(n, n, density=0.06, random_state=rng) + ss.diags(4 + rng.uniform(0, 1, n))
    a = a.tocsr()
    a.sort_indices()
    return a, rng.normal(size=n)


def test_full_restart_is_a_direct_solve():
    a, b = nonsymmetric(40, 1)
    x, it, res, tgt = O.gmres(O.Operator.csr(O.CSR.from_scipy(a)), b, tol=1e-14, restart=40,
                              maxiter=40)
    np.testing.assert_allclose(x, np.linalg.solve(a.toarray(), b), rtol=1e-10, atol=1e-12)
    assert it <= 40


def test_restarts_and_preconditioner_converge():
    a, b = nonsymmetric(150, 2)
    A = O.Operator.csr(O.CSR.from_scipy(a))
    for M in (None, O.Operator.diagonal(1 / a.diagonal())):
        x, it, res, tgt = O.gmres(A, b, M=M, tol=1e-10, restart=6, maxiter=300)
        assert res <= tgt and it > 6  # several cycles
        assert np.linalg.norm(b - a @ x) <= 2 * tgt


def test_maxiter_caps_the_steps():
    a, b = nonsymmetric(150, 3)
    x, it, res, tgt = O.gmres(O.Operator.csr(O.CSR.from_scipy(a)), b, tol=1e-14, restart=4,
                              maxiter=7)
    assert it == 7 and res > tgt
    # the residual norm reported is the true one of the returned x (to rounding)
    np.testing.assert_allclose(res, np.linalg.norm(b - a @ x), rtol=1e-6)
