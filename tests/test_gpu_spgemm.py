"""Device assembly of the smoothing operator (sparse.spgemm) against the
oracle's restatement of the reference's SciPy product, bit for bit, and an
FSAI built on it."""

import numpy as np
import pytest
import scipy.sparse as ss
import torch

from gpu_helpers import cuda, host_csr, oracle_csr, to_bsr, vec

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("side", [7, 13])
def test_device_biharmonic_assembly_bit_exact(oracle, side):
    from warp_preconditioners_gb300 import problems, sparse

    _, _, K, mass = problems.tet_cube(side)
    Kd = to_bsr(K)
    m = vec(mass)
    Q = sparse.spgemm(Kd, Kd, col_scale=1.0 / m, add_diag=1e-4 * m)
    Kc = oracle_csr(oracle, K)
    ref = oracle.spgemm(Kc, Kc, 1.0 / mass, 1e-4 * mass)
    off, col, val = host_csr(Q)
    np.testing.assert_array_equal(off, ref.offsets)
    np.testing.assert_array_equal(col, ref.columns)
    np.testing.assert_array_equal(val, ref.values)
    # Against this host's SciPy (which may fuse multiply-adds): within
    # rounding of the sum of absolute contributions |K| M^-1 |K| + alpha M.
    host = problems.biharmonic(K, mass, 1e-4)
    absq = (abs(K) @ ss.diags(1.0 / mass) @ abs(K) + ss.diags(1e-4 * mass)).tocsr()
    rows = np.repeat(np.arange(len(off) - 1), np.diff(off))
    scale = np.asarray(absq[rows, col.astype(np.int64)]).ravel()
    assert np.all(np.abs(val - host.data) <= 1e-14 * scale)


def test_plain_product_and_fsai_on_device_q(oracle):
    from warp_preconditioners_gb300 import FSAI, problems, sparse

    rng = np.random.default_rng(27)
    a = ss.random(300, 200, density=0.03, random_state=rng, format="csr")
    b = ss.random(200, 150, density=0.05, random_state=rng, format="csr")
    c = sparse.spgemm(to_bsr(a), to_bsr(b))
    ref = oracle.spgemm(oracle_csr(oracle, a), oracle_csr(oracle, b))
    off, col, val = host_csr(c)
    np.testing.assert_array_equal(off, ref.offsets)
    np.testing.assert_array_equal(col, ref.columns)
    np.testing.assert_array_equal(val, ref.values)
    # FSAI on the device-assembled Q equals the oracle's FSAI on its Q.
    _, _, K, mass = problems.tet_cube(8)
    Kd, m = to_bsr(K), vec(mass)
    Q = sparse.spgemm(Kd, Kd, col_scale=1.0 / m, add_diag=1e-4 * m)
    pre = FSAI(Q, max_row_size=8, kap_tolerance=1e-3)
    Kc = oracle_csr(oracle, K)
    g_or, _, _ = oracle.fsai(oracle.spgemm(Kc, Kc, 1.0 / mass, 1e-4 * mass), width=8, tol=1e-3)
    o2, c2, v2 = host_csr(pre.G)
    np.testing.assert_array_equal(c2, g_or.columns)
    np.testing.assert_array_equal(v2, g_or.values)
    with pytest.raises(ValueError):
        sparse.spgemm(to_bsr(a), to_bsr(a))
