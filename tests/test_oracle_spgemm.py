"""The oracle's sparse product against SciPy, which is what the reference
assembles the smoothing operator with (Q = alpha M + K M^-1 K on the host,
results/dirichlet-tuning/README.md:72-77).  On x86-64 SciPy's compiled loops
round every product and sum separately, so the oracle reproduces Q bit for
bit; elsewhere a compiler may fuse them, hence the tolerance branch."""

import platform

import numpy as np
import scipy.sparse as ss

from oracle import oracle as O
from warp_preconditioners_gb300 import problems

EXACT = platform.machine() in ("x86_64", "AMD64")


def check(c, ref):
    ref = ref.tocsr()
    ref.sort_indices()
    np.testing.assert_array_equal(c.offsets, ref.indptr)
    np.testing.assert_array_equal(c.columns, ref.indices)
    if EXACT:
        np.testing.assert_array_equal(c.values, ref.data)
    else:
        np.testing.assert_allclose(c.values, ref.data, rtol=1e-14, atol=0)


def test_biharmonic_assembly_matches_scipy():
    for side in (6, 11):
        _, _, K, mass = problems.tet_cube(side)
        Kc = O.CSR.from_scipy(K)
        check(O.spgemm(Kc, Kc, 1.0 / mass, 1e-4 * mass), problems.biharmonic(K, mass, 1e-4))


def test_plain_and_rectangular_products():
    rng = np.random.default_rng(18)
    a = ss.random(40, 30, density=0.15, random_state=rng, format="csr")
    b = ss.random(30, 25, density=0.2, random_state=rng, format="csr")
    a.sort_indices()
    b.sort_indices()
    check(O.spgemm(O.CSR.from_scipy(a), O.CSR.from_scipy(b)), a @ b)
    d = rng.uniform(0.5, 2.0, 30)
    check(O.spgemm(O.CSR.from_scipy(a), O.CSR.from_scipy(b), d), a @ ss.diags(d) @ b)


def test_cancellation_drops_exact_zeros():
    a = ss.csr_matrix(np.array([[1.0, 1.0], [0.0, 1.0]]))
    b = ss.csr_matrix(np.array([[1.0, 0.0], [-1.0, 1.0]]))
    c = O.spgemm(O.CSR.from_scipy(a), O.CSR.from_scipy(b))
    # row 0: (1*1 + 1*-1, 1*1) -> the zero at column 0 is dropped
    assert list(c.offsets) == [0, 1, 3]
    assert list(c.columns) == [1, 0, 1]
