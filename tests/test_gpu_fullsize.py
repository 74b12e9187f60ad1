"""Parity at the benchmark sizes: the GPU setup kernels against the oracle on
the full configurations, not only on small cases.

* The 70^3 smoothing system (343,000 unknowns, Q with ~21M entries): the
  FSAI factor at width 8, step 1 (every row) and at width 48, step 2 (a
  sample of rows: the first and last 1,000 and every 149th in between, each
  built by the oracle on its own, since every row of the reference's build
  is independent), supports and values bit for bit.
* The 64^3 block coupling K (x) C (262,144 block rows of 3 x 3): block
  Jacobi inverses, block ILU(0) with 3 factor sweeps, the scalarised FSAI
  (width 8, kap 3e-3, float32 factor), bit for bit; scalar Jacobi's apply at
  1e-14 relative.
"""

import numpy as np
import pytest
import torch

from gpu_helpers import cuda, host_csr, vec

pytestmark = pytest.mark.gpu

ALPHA = 1e-4


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.int64 if a.dtype == np.float64 else np.int32)


@pytest.fixture(scope="module")
def smoothing70():
    from warp_preconditioners_gb300 import problems

    verts, tets, K, mass = problems.tet_cube(70)
    return problems.biharmonic(K, mass, ALPHA)


@pytest.fixture(scope="module")
def coupling64():
    from warp_preconditioners_gb300 import problems

    bsr, _ = problems.kron_coupling(64, kappa=1e-6, seed=0)
    bsr.sort_indices()
    return bsr


def test_fsai_w8_step1_at_70cubed(oracle, smoothing70):
    from warp_preconditioners_gb300 import FSAI, from_scipy

    q = smoothing70
    pre = FSAI(from_scipy(q, cuda()), max_row_size=8, max_step_size=1, kap_tolerance=1e-3)
    g_or, gt_or, trunc = oracle.fsai(oracle.CSR(q.indptr, q.indices, q.data), width=8, step=1,
                                     tol=1e-3)
    for dev_m, host in ((pre.G, g_or), (pre.GT, gt_or)):
        off, col, val = host_csr(dev_m)
        np.testing.assert_array_equal(off, host.offsets)
        np.testing.assert_array_equal(col, host.columns)
        np.testing.assert_array_equal(_bits(val), _bits(host.values))
    assert pre.truncated_rows == trunc


def test_fsai_w48_step2_at_70cubed_sampled_rows(oracle, smoothing70):
    from warp_preconditioners_gb300 import FSAI, from_scipy

    q = smoothing70
    n = q.shape[0]
    pre = FSAI(from_scipy(q, cuda()), max_row_size=48, max_step_size=2, kap_tolerance=1e-3)
    off, col, val = host_csr(pre.G)
    rows = np.unique(np.concatenate([np.arange(1000), np.arange(n - 1000, n),
                                     np.arange(1000, n - 1000, 149)])).astype(np.int32)
    out, status = oracle.fsai_rows(oracle.CSR(q.indptr, q.indices, q.data), rows, width=48,
                                   step=2, tol=1e-3)
    assert status[2] == 0
    for r, (c, v) in zip(rows, out):
        np.testing.assert_array_equal(col[off[r]:off[r + 1]], c, err_msg=f"row {r}")
        np.testing.assert_array_equal(_bits(val[off[r]:off[r + 1]]), _bits(v),
                                      err_msg=f"row {r}")
    # The transpose is the exact transpose of the device factor.
    gt_off, gt_col, gt_val = host_csr(pre.GT)
    t = oracle.transpose(oracle.CSR(off, col, val))
    np.testing.assert_array_equal(gt_off, t.offsets)
    np.testing.assert_array_equal(gt_col, t.columns)
    np.testing.assert_array_equal(_bits(gt_val), _bits(t.values))


def _block_matrix(bsr):
    from warp_preconditioners_gb300.sparse import BsrMatrix

    nrow = bsr.shape[0] // 3
    return BsrMatrix(nrow, nrow, (3, 3), torch.as_tensor(bsr.indptr.astype(np.int32),
                                                          device=cuda()),
                     torch.as_tensor(bsr.indices.astype(np.int32), device=cuda()),
                     torch.as_tensor(np.ascontiguousarray(bsr.data), device=cuda()))


def test_block_jacobi_and_ilu0_at_64cubed(oracle, coupling64):
    from warp_preconditioners_gb300 import BlockILU0, BlockJacobi

    bsr = coupling64
    A = _block_matrix(bsr)
    nrow = A.nrow
    jac = BlockJacobi(A)
    inv, bad = oracle.block_diag_inverse(nrow, 3, bsr.indptr, bsr.indices, bsr.data)
    assert bad == 0
    np.testing.assert_array_equal(_bits(jac.inverse_diagonal.cpu().numpy()), _bits(inv))
    ilu = BlockILU0(A, factor_sweeps=3, solve_sweeps=3)
    fac, inv2, bad = oracle.bilu0_setup(nrow, 3, bsr.indptr, bsr.indices, bsr.data,
                                        factor_sweeps=3)
    assert bad == 0
    np.testing.assert_array_equal(_bits(ilu.factors.cpu().numpy()), _bits(fac))
    np.testing.assert_array_equal(_bits(ilu.inverse_diagonal.cpu().numpy()), _bits(inv2))
    rng = np.random.default_rng(0)
    x_np = rng.uniform(-1, 1, size=3 * nrow)
    z = torch.empty(3 * nrow, dtype=torch.float64, device=cuda())
    ilu.matvec(vec(x_np), vec(np.zeros_like(x_np)), z, 1.0, 0.0)
    want = oracle.bilu0_apply(nrow, 3, bsr.indptr, bsr.indices, fac, inv2, 3, x_np,
                              np.zeros_like(x_np), 1.0, 0.0)
    # 1e-9 of the largest entry: the 1e6-conditioned 3 x 3 inverse blocks
    # amplify the fused multiply-adds' rounding differences.
    np.testing.assert_allclose(z.cpu().numpy(), want, rtol=1e-9,
                               atol=1e-9 * np.abs(want).max())


def test_scalarised_fsai_at_64cubed(oracle, coupling64):
    from warp_preconditioners_gb300 import FSAI

    bsr = coupling64
    A = _block_matrix(bsr)
    pre = FSAI(A, max_row_size=8, kap_tolerance=3e-3, factor_dtype=torch.float32)
    sc = oracle.scalarize(A.nrow, 3, bsr.indptr, bsr.indices, bsr.data)
    g, gt, _ = oracle.fsai(sc, width=8, step=1, tol=3e-3, factor_dtype=np.float32)
    for dev_m, host in ((pre.G, g), (pre.GT, gt)):
        off, col, val = host_csr(dev_m)
        np.testing.assert_array_equal(off, host.offsets)
        np.testing.assert_array_equal(col, host.columns)
        np.testing.assert_array_equal(_bits(val), _bits(host.values))


def test_scalar_jacobi_on_3x3_blocks(coupling64):
    from warp_preconditioners_gb300 import linear

    bsr = coupling64
    A = _block_matrix(bsr)
    M = linear.preconditioner(A, "diag")
    n = 3 * A.nrow
    d = bsr.diagonal()
    rng = np.random.default_rng(1)
    x_np, y_np = rng.uniform(-1, 1, size=n), rng.uniform(-1, 1, size=n)
    z = torch.empty(n, dtype=torch.float64, device=cuda())
    M.matvec(vec(x_np), vec(y_np), z, 0.7, -0.2)
    want = 0.7 * (x_np / d) - 0.2 * y_np
    np.testing.assert_allclose(z.cpu().numpy(), want, rtol=1e-14, atol=1e-15)
