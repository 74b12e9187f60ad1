"""Sparse products, factored biharmonic, block Jacobi, block ILU(0), block FSAI on
the GPU against the oracle and the reference's known answers."""

import numpy as np
import pytest
import scipy.sparse as ss
import torch

from gpu_helpers import cuda, oracle_csr, to_bsr, vec

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("lanes", [1, 2, 4, 8, 16, 32])
def test_sparse_operator_rows_aliases_and_graph(dtype, lanes):
    # tests/test_sparse_operator.py:12-47: irregular rows, empty row 0.
    from warp_preconditioners_gb300 import SparseOperator

    rng = np.random.default_rng(91)
    a = ss.random(67, 67, density=0.12, random_state=rng, format="csr")
    a.data = rng.normal(size=a.nnz)
    a = a.tolil()
    a[0, :] = 0
    a = a.tocsr()
    A = SparseOperator(to_bsr(a, dtype), row_lanes=lanes)
    rtol, atol = (2e-5, 2e-6) if dtype == torch.float32 else (1e-12, 1e-12)
    for alias in ["none", "xz", "yz", "xyz"]:
        x = vec(rng.normal(size=67), dtype)
        y = x if alias == "xyz" else vec(rng.normal(size=67), dtype)
        z = x if alias in ["xz", "xyz"] else y if alias == "yz" else torch.empty_like(x)
        ref = 0.7 * (a @ x.cpu().double().numpy()) - 0.3 * y.cpu().double().numpy()
        A.matvec(x, y, z, 0.7, -0.3)
        np.testing.assert_allclose(z.cpu().double().numpy(), ref, rtol=rtol, atol=atol)
    x = vec(rng.normal(size=67), dtype)
    y = torch.full_like(x, float("nan"))
    z = torch.empty_like(x)
    A.matvec(x, y, z, 1.0, 0.0)
    np.testing.assert_allclose(z.cpu().double().numpy(), a @ x.cpu().double().numpy(), rtol=rtol,
                               atol=atol)
    x.fill_(float("nan"))
    y.fill_(2.0)
    A.matvec(x, y, z, 0.0, 0.5)
    np.testing.assert_array_equal(z.cpu().numpy(), 1.0)
    x.fill_(1.0)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        A.matvec(x, y, z, 1.0, 0.0)
    z.zero_()
    graph.replay()
    torch.cuda.synchronize()
    np.testing.assert_allclose(z.cpu().double().numpy(), a @ np.ones(67), rtol=rtol, atol=atol)


def test_sparse_operator_matches_oracle_bsr(oracle):
    from warp_preconditioners_gb300 import SparseOperator, problems

    bsr, _ = problems.kron_coupling(6, 1e-6)
    bsr.sort_indices()
    A = SparseOperator(to_bsr(bsr.toarray(), block=3))
    rng = np.random.default_rng(3)
    x, y = rng.normal(size=(2, bsr.shape[0]))
    z = torch.empty(bsr.shape[0], dtype=torch.float64, device=cuda())
    A.matvec(vec(x), vec(y), z, 1.3, 0.4)
    ref = oracle.bsr_spmv(bsr.shape[0] // 3, 3, bsr.indptr, bsr.indices, bsr.data, x, y, 1.3, 0.4)
    np.testing.assert_allclose(z.cpu().numpy(), ref, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("mass_weight", [0.0, 0.15])
def test_factored_operator_and_rhs(golden, dtype, mass_weight):
    # tests/test_squared_laplacian.py:12-63
    from warp_preconditioners_gb300 import SquaredLaplacianOperator

    d = golden("sqlap.npz")
    npdt = np.float64 if dtype == torch.float64 else np.float32
    A = SquaredLaplacianOperator(to_bsr(d["lap"], dtype), vec(d["mass"].astype(npdt), dtype),
                                 torch.as_tensor(d["free"], device=cuda()), row_lanes=4,
                                 mass_weight=mass_weight)
    reduced = d[f"reduced_w{mass_weight}"]
    rtol, atol = (3e-5, 3e-6) if dtype == torch.float32 else (1e-12, 1e-12)
    rng = np.random.default_rng(27)
    nf = len(d["free"])
    for alias in ["none", "xz", "yz", "xyz"]:
        x = vec(rng.normal(size=nf), dtype)
        y = x if alias == "xyz" else vec(rng.normal(size=nf), dtype)
        z = x if alias in ["xz", "xyz"] else y if alias == "yz" else torch.empty_like(x)
        expected = 0.7 * (reduced @ x.cpu().double().numpy()) - 0.2 * y.cpu().double().numpy()
        A.matvec(x, y, z, 0.7, -0.2)
        np.testing.assert_allclose(z.cpu().double().numpy(), expected, rtol=rtol, atol=atol)
    bw = vec(d[f"bc_w{mass_weight}"].astype(npdt), dtype)
    result = A.rhs(bw)
    np.testing.assert_allclose(result.cpu().double().numpy(), d[f"rhs_w{mass_weight}"], rtol=rtol,
                               atol=atol)
    x = torch.ones(nf, dtype=dtype, device=cuda())
    y = torch.full_like(x, float("nan"))
    z = torch.empty_like(x)
    A.matvec(x, y, z, 1.0, 0.0)
    np.testing.assert_allclose(z.cpu().double().numpy(), reduced @ np.ones(nf), rtol=rtol,
                               atol=atol)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        A.matvec(x, y, z, 1.0, 0.0)
        A.rhs(bw, out=result)
    z.zero_()
    graph.replay()
    torch.cuda.synchronize()
    np.testing.assert_allclose(z.cpu().double().numpy(), reduced @ np.ones(nf), rtol=rtol,
                               atol=atol)


def test_squared_validation():
    from warp_preconditioners_gb300 import SquaredLaplacianOperator

    L = to_bsr(np.eye(5))
    mass = torch.ones(5, dtype=torch.float64, device=cuda())
    for weight in [-1, float("nan"), float("inf")]:
        with pytest.raises(ValueError, match="mass_weight"):
            SquaredLaplacianOperator(L, mass, torch.tensor([1, 2], dtype=torch.int32,
                                                           device=cuda()), mass_weight=weight)
    for free in [[0, 0], [0, 5], [-1, 2]]:
        with pytest.raises(ValueError, match="free_indices"):
            SquaredLaplacianOperator(L, mass, torch.tensor(free, dtype=torch.int32, device=cuda()))
    with pytest.raises(ValueError, match="mass entries"):
        SquaredLaplacianOperator(L, torch.zeros_like(mass),
                                 torch.tensor([1, 2], dtype=torch.int32, device=cuda()))


def test_tet_cube_factored_equals_assembled(oracle):
    from warp_preconditioners_gb300 import SparseOperator, SquaredLaplacianOperator, problems

    _, _, K, mass = problems.tet_cube(10)
    q = problems.biharmonic(K, mass, 1e-4)
    n = K.shape[0]
    fact = SquaredLaplacianOperator(to_bsr(K), vec(mass), torch.arange(n, dtype=torch.int32,
                                                                       device=cuda()),
                                    mass_weight=1e-4)
    asm = SparseOperator(to_bsr(q))
    x = vec(np.random.default_rng(0).normal(size=n))
    z1 = torch.empty_like(x)
    z2 = torch.empty_like(x)
    fact.matvec(x, x, z1, 1.0, 0.0)
    asm.matvec(x, x, z2, 1.0, 0.0)
    np.testing.assert_allclose(z1.cpu().numpy(), z2.cpu().numpy(), rtol=1e-10, atol=1e-12)
    ref = oracle.Operator.sqlap(oracle_csr(oracle, K), mass, 1e-4).apply(x.cpu().numpy(),
                                                                         np.zeros(n), 1.0, 0.0)
    np.testing.assert_allclose(z1.cpu().numpy(), ref, rtol=1e-12, atol=1e-15)


def test_identity_free_shares_one_copy_of_L(oracle):
    # With every vertex free in index order one stored copy of L serves the
    # forward and backward products, the forward one walking its slices in
    # reverse.  At 56^3 (5,488 slices) the walk has a partial last pass.
    # The same system with its unknowns listed in a random order takes the
    # two-copy path; both must give the oracle's product, and the two paths
    # the same vector up to the reordering.
    from warp_preconditioners_gb300 import SquaredLaplacianOperator, from_scipy, problems

    _, _, K, mass = problems.tet_cube(56)
    n = K.shape[0]
    dev = cuda()
    Kd, md = from_scipy(K, dev), vec(mass)
    rng = np.random.default_rng(5)
    x_np = rng.normal(size=n)
    perm = rng.permutation(n).astype(np.int32)
    ident = SquaredLaplacianOperator(Kd, md, torch.arange(n, dtype=torch.int32, device=dev),
                                     mass_weight=1e-4)
    permuted = SquaredLaplacianOperator(Kd, md, torch.as_tensor(perm, device=dev),
                                        mass_weight=1e-4)
    x = vec(x_np)
    z1 = torch.empty_like(x)
    ident.matvec(x, x, z1, 1.0, 0.0)
    z1b = torch.empty_like(x)
    ident.matvec(x, x, z1b, 1.0, 0.0)
    assert torch.equal(z1, z1b)
    xp = vec(x_np[perm])
    z2 = torch.empty_like(xp)
    permuted.matvec(xp, xp, z2, 1.0, 0.0)
    ref = oracle.Operator.sqlap(oracle_csr(oracle, K), mass, 1e-4).apply(x_np, np.zeros(n),
                                                                         1.0, 0.0)
    scale = np.abs(ref).max()
    np.testing.assert_allclose(z1.cpu().numpy(), ref, rtol=1e-12, atol=1e-14 * scale)
    np.testing.assert_allclose(z2.cpu().numpy(), z1.cpu().numpy()[perm], rtol=1e-12,
                               atol=1e-14 * scale)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("size", [1, 2, 3, 4])
def test_block_factors_and_aliases(oracle, dtype, size):
    # tests/test_indefinite.py:12-53
    from warp_preconditioners_gb300 import BlockILU0, BlockJacobi

    rng = np.random.default_rng(61)
    n = 5
    blocks = rng.normal(size=(n, n, size, size)) * 0.03
    for i in range(n):
        blocks[i, i] = np.diag(np.arange(1, size + 1) * np.where(np.arange(size) % 2, -1.0, 1.0))
    a = blocks.transpose(0, 2, 1, 3).reshape(n * size, n * size)
    A = to_bsr(a, dtype, block=size)
    pre = BlockILU0(A, factor_sweeps=2 * n + 2, solve_sweeps=n)
    jac = BlockJacobi(A)
    expected = np.linalg.inv(a)
    tol = dict(rtol=2e-5, atol=1e-6) if dtype == torch.float32 else dict(rtol=1e-12, atol=1e-12)
    for alias in ["none", "xz", "yz", "xyz"]:
        x = vec(rng.normal(size=(n, size)), dtype)
        y = x if alias == "xyz" else vec(rng.normal(size=(n, size)), dtype)
        z = x if alias in ["xz", "xyz"] else y if alias == "yz" else torch.empty_like(x)
        target = 0.7 * (expected @ x.cpu().double().numpy().ravel()) - \
            0.2 * y.cpu().double().numpy().ravel()
        pre.matvec(x, y, z, 0.7, -0.2)
        np.testing.assert_allclose(z.cpu().double().numpy().ravel(), target, **tol)
    x = vec(rng.normal(size=(n, size)), dtype)
    y = torch.empty_like(x)
    jac.matvec(x, y, y, 1.0, 0.0)
    target = np.stack([np.linalg.solve(blocks[i, i], x.cpu().double().numpy()[i])
                       for i in range(n)])
    np.testing.assert_allclose(y.cpu().double().numpy(), target, rtol=1e-5, atol=1e-6)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        pre.matvec(x, y, y, 1.0, 0.0)
    graph.replay()
    torch.cuda.synchronize()
    np.testing.assert_allclose(y.cpu().double().numpy().ravel(),
                               expected @ x.cpu().double().numpy().ravel(), **tol)


def test_ilu0_factors_known_answer_and_linearity(golden):
    # tests/test_indefinite.py:148-192
    from warp_preconditioners_gb300 import BlockILU0

    d = golden("ilu0_recurrence.npz")
    A = to_bsr(d["a"], block=2)
    n = 9
    pre = BlockILU0(A, factor_sweeps=2 * n + 2, solve_sweeps=3)
    off, col = A.offsets.cpu().numpy(), A.columns.cpu().numpy()
    factors = pre.factors.cpu().numpy()
    lookup = {(int(r), int(c)): f for r, c, f in zip(d["rows"], d["cols"], d["factors"])}
    assert len(factors) == len(lookup)
    for i in range(n):
        for e in range(off[i], off[i + 1]):
            np.testing.assert_allclose(factors[e], lookup[(i, int(col[e]))], rtol=1e-12,
                                       atol=1e-12)
    rng = np.random.default_rng(83)

    def apply(v):
        x = vec(v)
        y = torch.empty_like(x)
        pre.matvec(x, y, y, 1.0, 0.0)
        return y.cpu().numpy()

    x, y = rng.normal(size=(2, n, 2))
    np.testing.assert_allclose(apply(0.3 * x + 0.7 * y), 0.3 * apply(x) + 0.7 * apply(y),
                               rtol=1e-12, atol=1e-12)
    xw = torch.full((n, 2), float("nan"), dtype=torch.float64, device=cuda())
    yw = vec(y)
    pre.matvec(xw, yw, xw, 0.0, 0.7)
    np.testing.assert_allclose(xw.cpu().numpy(), 0.7 * y)


def test_block_pivot_errors_and_update_rollback():
    from warp_preconditioners_gb300 import BlockJacobi

    with pytest.raises(ValueError, match="pivot"):
        BlockJacobi(to_bsr(np.diag([1.0, 0.0]), block=2))
    rng = np.random.default_rng(46)
    r = rng.normal(size=(6, 6))
    a = r @ r.T + np.eye(6)
    pre = BlockJacobi(to_bsr(a, block=3))
    saved = pre.inverse_diagonal.clone()
    singular = to_bsr(np.diag([1.0, 1.0, 1.0, 1.0, 1.0, 0.0]), block=3)
    with pytest.raises(ValueError, match="pivot"):
        pre.update(singular)
    torch.testing.assert_close(pre.inverse_diagonal, saved)


def test_block_ilu0_bsr_matches_oracle(oracle):
    from warp_preconditioners_gb300 import BlockILU0, problems

    bsr, _ = problems.kron_coupling(8, 1e-6)
    bsr.sort_indices()
    nrow = bsr.shape[0] // 3
    pre = BlockILU0(to_bsr(bsr.toarray(), block=3), factor_sweeps=3, solve_sweeps=3)
    f_or, inv_or, bad = oracle.bilu0_setup(nrow, 3, bsr.indptr, bsr.indices, bsr.data,
                                           factor_sweeps=3)
    assert bad == 0
    np.testing.assert_allclose(pre.factors.cpu().numpy(), f_or, rtol=1e-11, atol=1e-12)
    x = np.random.default_rng(1).normal(size=bsr.shape[0])
    z = torch.empty(bsr.shape[0], dtype=torch.float64, device=cuda())
    pre.matvec(vec(x), vec(x), z, 1.0, 0.0)
    ref = oracle.bilu0_apply(nrow, 3, bsr.indptr, bsr.indices, f_or, inv_or, 3, x,
                             np.zeros_like(x), 1.0, 0.0)
    # C = R diag(1, 1, 1e-6) R^T: the inverse blocks amplify summation-order
    # differences by about 1e6, so agreement is to ~1e-16 * 1e6 * sweeps.
    np.testing.assert_allclose(z.cpu().numpy(), ref, rtol=1e-7, atol=1e-9)


@pytest.mark.parametrize("blocks", [1, 2, 4])
@pytest.mark.parametrize("bs", [2, 3])
def test_block_fsai_principal_inverse(oracle, bs, blocks):
    # tests/test_fsai_candidates.py:15-52
    from warp_preconditioners_gb300 import BlockFSAI, BsrBlockFSAI

    rng = np.random.default_rng(712)
    n = 4 * bs
    r = rng.normal(size=(n, n))
    a = r @ r.T + np.eye(n)
    s = np.geomspace(0.01, 100, n)
    a *= s[:, None] * s[None, :]
    A = to_bsr(a, block=bs)
    for factory in (BlockFSAI, BsrBlockFSAI):
        pre = factory(A, max_blocks=blocks, factor_dtype=torch.float64)
        g = pre.G.dense()
        assert np.linalg.eigvalsh(g.T @ g).min() > 0
        for i in range(4):
            row = g[bs * i:bs * (i + 1)]
            support = np.flatnonzero(np.any(row != 0, axis=0))
            rhs = np.zeros((len(support), bs))
            rhs[-bs:, :] = np.eye(bs)
            z = np.linalg.solve(a[np.ix_(support, support)], rhs)
            expected = np.linalg.solve(np.linalg.cholesky(z[-bs:, :]), z.T)
            np.testing.assert_allclose(row[:, support], expected, rtol=2e-11, atol=1e-10)
            np.testing.assert_allclose(row @ a @ row.T, np.eye(bs), atol=2e-12)
        if blocks == 4:
            np.testing.assert_allclose(g.T @ g, np.linalg.inv(a), rtol=2e-11, atol=1e-10)
        x = vec(rng.normal(size=(4, bs)))
        expected = 0.7 * g.T @ g @ x.cpu().numpy().ravel() - 0.2 * x.cpu().numpy().ravel()
        pre.matvec(x, x, x, 0.7, -0.2)
        np.testing.assert_allclose(x.cpu().numpy().ravel(), expected, rtol=2e-11, atol=1e-10)


def test_block_fsai_matches_oracle_on_coupling(oracle):
    from warp_preconditioners_gb300 import BsrBlockFSAI, problems

    bsr, _ = problems.kron_coupling(6, 1e-6)
    bsr.sort_indices()
    nrow = bsr.shape[0] // 3
    pre = BsrBlockFSAI(to_bsr(bsr.toarray(), block=3), max_blocks=2, factor_dtype=torch.float64)
    cols, vals, _, bad = oracle.block_fsai_setup(nrow, 3, 2, bsr.indptr, bsr.indices, bsr.data)
    g_or = oracle.fsai_pack(bsr.shape[0], 6, cols, vals)
    np.testing.assert_array_equal(pre.G.offsets.cpu().numpy(), g_or.offsets)
    np.testing.assert_array_equal(pre.G.columns.cpu().numpy(), g_or.columns)
    np.testing.assert_allclose(pre.G.values.cpu().numpy(), g_or.values, rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(pre.B.dense(), pre.G.dense(), rtol=0, atol=0)
