"""Every sliced-ELL product variant gives the same bits: products, fused dot
products and whole preconditioned solves, on irregular rows (empty rows,
lengths 0..40, length-sorted windows) and on the benchmark's operator.
GBPC_SPMV_VARIANT fixes the variant the autotuner would pick."""

import os

import numpy as np
import pytest
import scipy.sparse as ss
import torch

from gpu_helpers import cuda, to_bsr, vec

pytestmark = pytest.mark.gpu

VARIANTS = range(6)


@pytest.fixture
def variant_env():
    old = os.environ.get("GBPC_SPMV_VARIANT")
    yield
    if old is None:
        os.environ.pop("GBPC_SPMV_VARIANT", None)
    else:
        os.environ["GBPC_SPMV_VARIANT"] = old


def irregular(n, seed):
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 41, size=n)
    lens[rng.random(n) < 0.05] = 0
    rows = np.repeat(np.arange(n), lens)
    cols = rng.integers(0, n, size=rows.size)
    a = ss.csr_matrix((rng.normal(size=rows.size), (rows, cols)), shape=(n, n))
    a.sum_duplicates()
    return a


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_products_identical_across_variants(variant_env, dtype):
    from warp_preconditioners_gb300 import SparseOperator

    a = irregular(20011, 5)
    rng = np.random.default_rng(6)
    x, y = vec(rng.normal(size=a.shape[0]), dtype), vec(rng.normal(size=a.shape[0]), dtype)
    out = []
    for v in VARIANTS:
        os.environ["GBPC_SPMV_VARIANT"] = str(v)
        A = SparseOperator(to_bsr(a, dtype))
        z = torch.empty_like(x)
        A.matvec(x, y, z, 0.7, -0.3)
        z2 = torch.empty_like(x)
        A.matvec(x, y, z2, 1.0, 0.0)
        out.append((z.cpu().numpy(), z2.cpu().numpy()))
    ref = 0.7 * (a @ x.cpu().double().numpy()) - 0.3 * y.cpu().double().numpy()
    rtol, atol = (1e-4, 1e-4) if dtype == torch.float32 else (1e-12, 1e-12)
    np.testing.assert_allclose(out[0][0], ref, rtol=rtol, atol=atol)
    for v in VARIANTS:
        np.testing.assert_array_equal(out[v][0], out[0][0])
        np.testing.assert_array_equal(out[v][1], out[0][1])


def test_solves_identical_across_variants(variant_env):
    # A solve reads every fused dot product's bits: equal iterates after 60
    # PCG iterations on the factored biharmonic operator mean equal dots.
    from warp_preconditioners_gb300 import FSAI, SquaredLaplacianOperator, linear, problems

    _, _, K, mass = problems.tet_cube(20)
    q = problems.biharmonic(K, mass, 1e-4)
    b = vec(np.random.default_rng(7).normal(size=K.shape[0]))
    runs = []
    for v in VARIANTS:
        os.environ["GBPC_SPMV_VARIANT"] = str(v)
        free = torch.arange(K.shape[0], dtype=torch.int32, device=cuda())
        A = SquaredLaplacianOperator(to_bsr(K), vec(mass), free, mass_weight=1e-4)
        pre = FSAI(to_bsr(q), max_row_size=8)
        x = torch.zeros_like(b)
        nit, rr, _ = linear.cg(A, b, x, tol=1e-30, M=pre, maxiter=60, check_every=0)
        runs.append((int(nit.item()), float(rr.item()), x.cpu().numpy()))
    assert runs[0][0] == 60
    for v in VARIANTS:
        assert runs[v][0] == runs[0][0] and runs[v][1] == runs[0][1]
        np.testing.assert_array_equal(runs[v][2], runs[0][2])


@pytest.mark.parametrize("shape", ["one_row", "n31", "n32", "n33", "empty_rows", "wide"])
def test_edge_shapes_across_variants(variant_env, shape):
    from warp_preconditioners_gb300 import SparseOperator

    rng = np.random.default_rng(11)
    if shape == "one_row":
        a = ss.csr_matrix(np.array([[2.5]]))
    elif shape.startswith("n"):
        n = int(shape[1:])
        a = ss.random(n, n, density=0.3, random_state=rng, format="csr") + ss.eye(n)
    elif shape == "empty_rows":
        a = ss.csr_matrix((300, 300))
    else:  # rows of 64 entries: many more slices than warps, each several chunks
        n = 200_000
        rows = np.repeat(np.arange(n), 64)
        cols = (rows + rng.integers(0, 4096, size=rows.size)) % n
        a = ss.csr_matrix((rng.normal(size=rows.size), (rows, cols)), shape=(n, n))
        a.sum_duplicates()
    a = ss.csr_matrix(a)
    x, y = vec(rng.normal(size=a.shape[0])), vec(rng.normal(size=a.shape[0]))
    ref = 1.5 * (a @ x.cpu().numpy()) + 0.5 * y.cpu().numpy()
    out = []
    for v in VARIANTS:
        os.environ["GBPC_SPMV_VARIANT"] = str(v)
        A = SparseOperator(to_bsr(a))
        z = torch.empty_like(x)
        A.matvec(x, y, z, 1.5, 0.5)
        out.append(z.cpu().numpy())
    np.testing.assert_allclose(out[0], ref, rtol=1e-12, atol=1e-12)
    for v in VARIANTS:
        np.testing.assert_array_equal(out[v], out[0])


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_unit_scaling_products_equal_general_path(variant_env, dtype):
    # alpha = 1, beta = 0 runs the instantiation that issues no scaling or y
    # term; alpha = 1, beta = 1 with y = 0 runs the run-time-flag path and
    # adds exact zeros.  Every variant must give the same bits both ways.
    from warp_preconditioners_gb300 import FSAI, SparseOperator, problems

    a = irregular(20011, 9)
    q = problems.laplacian_2d(40)
    rng = np.random.default_rng(10)
    for v in VARIANTS:
        os.environ["GBPC_SPMV_VARIANT"] = str(v)
        for op, n in ((SparseOperator(to_bsr(a, dtype)), a.shape[0]),
                      (FSAI(to_bsr(q, dtype), max_row_size=8), q.shape[0])):
            x = vec(rng.normal(size=n), dtype)
            zeros = torch.zeros_like(x)
            z_unit, z_gen = torch.empty_like(x), torch.empty_like(x)
            op.matvec(x, x, z_unit, 1.0, 0.0)
            op.matvec(x, zeros, z_gen, 1.0, 1.0)
            np.testing.assert_array_equal(z_unit.cpu().numpy(), z_gen.cpu().numpy())


@pytest.mark.parametrize("block", [2, 3])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_blocked_products_identical_across_variants(variant_env, block, dtype):
    # Variant 4 on blocked rows is the pipelined blocked kernel; it must give
    # the one-slice blocked kernel's bits (rows of 0..14 blocks, empty rows).
    from warp_preconditioners_gb300 import SparseOperator

    rng = np.random.default_rng(12 + block)
    nb = 12007
    lens = rng.integers(0, 15, size=nb)
    rows = np.repeat(np.arange(nb), lens)
    cols = rng.integers(0, nb, size=rows.size)
    blocks = ss.csr_matrix((np.ones(rows.size), (rows, cols)), shape=(nb, nb))
    blocks.sum_duplicates()
    dense_pattern = ss.kron(blocks, np.ones((block, block)), format="csr")
    a = dense_pattern.multiply(rng.normal(size=dense_pattern.shape[0])[:, None]).tocsr()
    a.data = rng.normal(size=a.nnz)
    n = a.shape[0]
    x, y = vec(rng.normal(size=n), dtype), vec(rng.normal(size=n), dtype)
    out = {}
    for v in (0, 4):
        os.environ["GBPC_SPMV_VARIANT"] = str(v)
        A = SparseOperator(to_bsr(a, dtype, block))
        z1, z2 = torch.empty_like(x), torch.empty_like(x)
        A.matvec(x, y, z1, 0.7, -0.3)
        A.matvec(x, y, z2, 1.0, 0.0)
        out[v] = (z1.cpu().numpy(), z2.cpu().numpy())
    ref = 0.7 * (a @ x.cpu().double().numpy()) - 0.3 * y.cpu().double().numpy()
    rtol, atol = (1e-4, 1e-4) if dtype == torch.float32 else (1e-12, 1e-12)
    np.testing.assert_allclose(out[0][0], ref, rtol=rtol, atol=atol)
    for k in range(2):
        np.testing.assert_array_equal(out[4][k], out[0][k])


def test_blocked_solves_identical_across_variants(variant_env):
    # Fixed-iteration block-Jacobi CG on the K (x) C coupling: equal iterates
    # mean equal fused dots on 3 x 3 blocks.
    from warp_preconditioners_gb300 import BlockJacobi, SparseOperator, linear, problems

    bsr, _ = problems.kron_coupling(24, 1e-6)
    b = vec(np.random.default_rng(13).normal(size=bsr.shape[0]))
    xs = []
    for v in (0, 4):
        os.environ["GBPC_SPMV_VARIANT"] = str(v)
        A = SparseOperator(to_bsr(bsr, block=3))
        M = BlockJacobi(to_bsr(bsr, block=3))
        x = torch.zeros_like(b)
        nit, _, _ = linear.cg(A, b, x, tol=1e-30, M=M, maxiter=40, check_every=0)
        assert int(nit.item()) == 40
        xs.append(x.cpu().numpy())
    np.testing.assert_array_equal(xs[0], xs[1])
