"""Oracle fixed-support refit (fsai_reuse.py:75-149) against the known
answers of the reference's tests/test_updates.py: every refit row is the
normalised local solve z / sqrt(z_i) on its support, a full pattern gives
G^T G = A^-1, and invalid matrices are counted, not published."""

import numpy as np
import pytest
import scipy.sparse as ss

from oracle import oracle as O


def spd12(seed=48):
    r = np.random.default_rng(seed).normal(size=(12, 12))
    return r @ r.T + np.eye(12) * 3


@pytest.mark.parametrize("step", [1, 3])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_refit_rows_are_local_solves(step, dtype):
    a = spd12()
    A = O.CSR.from_scipy(ss.csr_matrix(a), dtype)
    g, _, _ = O.fsai(A, width=5, step=step)
    b = a + np.diag(np.arange(12.0))
    B = O.CSR.from_scipy(ss.csr_matrix(b), dtype)
    vals, bad_diag, bad_rows = O.fsai_refit(B, g)
    assert bad_diag == 0 and bad_rows == 0
    rtol = 1e-11 if dtype == np.float64 else 2e-4
    for i in range(12):
        lo, hi = g.offsets[i], g.offsets[i + 1]
        support = g.columns[lo:hi]
        assert support[-1] == i  # diagonal last
        e = np.zeros(len(support))
        e[-1] = 1
        z = np.linalg.solve(b[np.ix_(support, support)], e)
        np.testing.assert_allclose(vals[lo:hi], z / np.sqrt(z[-1]), rtol=rtol, atol=rtol * 1e-3)


def test_full_pattern_refit_is_exact_inverse():
    a = spd12()
    A = O.CSR.from_scipy(ss.csr_matrix(a))
    g, _, _ = O.fsai(A, width=12, tol=0.0)
    b = a + 0.5 * np.eye(12)
    vals, bd, br = O.fsai_refit(O.CSR.from_scipy(ss.csr_matrix(b)), g)
    assert bd == br == 0
    G = ss.csr_matrix((vals, g.columns, g.offsets), shape=(12, 12)).toarray()
    np.testing.assert_allclose(G.T @ G, np.linalg.inv(b), rtol=1e-10, atol=1e-13)


def test_refit_of_the_source_matches_the_build():
    # Same values: the refit reproduces the adaptive build's factor up to
    # rounding (the build borders its Cholesky, the refit factors afresh).
    a = spd12(7)
    A = O.CSR.from_scipy(ss.csr_matrix(a))
    g, _, _ = O.fsai(A, width=6, step=2)
    vals, bd, br = O.fsai_refit(A, g)
    assert bd == br == 0
    np.testing.assert_allclose(vals, g.values, rtol=1e-12, atol=1e-15)


def test_float32_storage_is_the_rounded_float64_refit():
    a = spd12()
    A = O.CSR.from_scipy(ss.csr_matrix(a))
    g, _, _ = O.fsai(A, width=5)
    v64, _, _ = O.fsai_refit(A, g)
    v32, _, _ = O.fsai_refit(A, g, factor_dtype=np.float32)
    assert v32.dtype == np.float32
    np.testing.assert_array_equal(v32, v64.astype(np.float32))


def test_invalid_matrices_are_counted():
    a = spd12()
    A = O.CSR.from_scipy(ss.csr_matrix(a))
    g, _, _ = O.fsai(A, width=5)
    zero = O.CSR(A.offsets, A.columns, np.zeros_like(A.values))
    _, bd, br = O.fsai_refit(zero, g)
    assert bd == 12 and br == 12
    # Indefinite local support: a 2x2 principal block with |a_ij| > sqrt(a_ii a_jj).
    c = np.eye(12) * 2.0
    c[1, 0] = c[0, 1] = 3.0
    C = O.CSR.from_scipy(ss.csr_matrix(c + 1e-3 * np.eye(12)))
    gfull, _, _ = O.fsai(O.CSR.from_scipy(ss.csr_matrix(np.eye(12) * 2 + 0.1 * (
        np.eye(12, k=1) + np.eye(12, k=-1)))), width=3)
    _, bd, br = O.fsai_refit(C, gfull)
    assert bd == 0 and br >= 1
