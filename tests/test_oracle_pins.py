"""Pin the CPU oracle to the reference's known answers (no GPU).

Each case restates an assertion of the reference's own tests against the
fixtures in tests/golden/ (generated by tests/golden/make_golden.py with dense
NumPy, independently of the oracle).
"""

import numpy as np
import pytest
import scipy.sparse as ss


def scalar_from_blocks(o, a, b, dtype=np.float64):
    """Scalar CSR of `a` seen through b x b blocks (stored zeros kept)."""
    bsr = ss.bsr_matrix(ss.csr_matrix(a), blocksize=(b, b))
    bsr.sort_indices()
    return o.scalarize(a.shape[0] // b, b, bsr.indptr, bsr.indices, bsr.data.astype(dtype))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("step", [1, 3])
@pytest.mark.parametrize("tol", [0.0, 0.003, 0.1])
def test_fsai_matches_independent_greedy_search(oracle, golden, dtype, step, tol):
    # tests/test_fsai.py:125-169 with 3x3 blocks holding stored zeros.
    data = golden("fsai_greedy.npz")
    a = data["a"]
    scalar = scalar_from_blocks(oracle, a, 3, dtype)
    g, _, _ = oracle.fsai(scalar, width=8, step=step, tol=tol)
    dense = g.to_scipy().toarray().astype(np.float64)
    expected = data[f"g_tol{tol}_step{step}"]
    np.testing.assert_array_equal(dense != 0, expected != 0)
    rtol, atol = (3e-5, 1e-6) if dtype == np.float32 else (1e-10, 1e-13)
    np.testing.assert_allclose(dense, expected, rtol=rtol, atol=atol)


@pytest.mark.parametrize("step", [2, 3])
def test_fsai_path_graph(oracle, golden, step):
    # tests/test_fsai.py:189-203
    data = golden("fsai_path.npz")
    g, _, _ = oracle.fsai(oracle.CSR.from_scipy(data["a"]), width=8, step=step, tol=0.0)
    np.testing.assert_array_equal(np.diff(g.offsets), data["counts"])
    np.testing.assert_allclose(g.to_scipy().toarray(), data["g"], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("step", [1, 3])
def test_fsai_full_pattern_is_exact_inverse(oracle, golden, step):
    # tests/test_fsai.py:36-51 and :206-213
    data = golden("fsai_full.npz")
    g, gt, _ = oracle.fsai(oracle.CSR.from_scipy(data["a8"]), width=8, step=step, tol=0.0)
    d = g.to_scipy().toarray()
    np.testing.assert_allclose(d.T @ d, data["inv8"], rtol=1e-10, atol=1e-12)
    assert np.allclose(d, np.tril(d))
    z = oracle.fsai_apply(g, gt, data["x8"], data["y8"], 1.7, -0.3)
    np.testing.assert_allclose(z, 1.7 * d.T @ d @ data["x8"] - 0.3 * data["y8"], rtol=1e-10)
    g32, _, _ = oracle.fsai(oracle.CSR.from_scipy(data["a32"]), width=32, step=3, tol=0.0)
    np.testing.assert_array_equal(np.diff(g32.offsets), np.arange(1, 33))
    d32 = g32.to_scipy().toarray()
    np.testing.assert_allclose(d32.T @ d32, data["inv32"], rtol=1e-12, atol=1e-15)


def test_fsai_local_solves_under_scaling(oracle, golden):
    # tests/test_fsai.py:73-90
    a = golden("fsai_scaled.npz")["a"]
    g, _, _ = oracle.fsai(oracle.CSR.from_scipy(a), width=5, tol=0.0)
    d = g.to_scipy().toarray()
    assert np.count_nonzero(d, axis=1).max() <= 5
    assert np.linalg.eigvalsh(d.T @ d).min() > 0
    for i in range(len(a)):
        support = np.flatnonzero(d[i])
        e = np.zeros(len(support))
        e[-1] = 1
        ref = np.linalg.solve(a[np.ix_(support, support)], e)
        ref /= np.sqrt(ref[-1])
        np.testing.assert_allclose(d[i, support], ref, rtol=1e-10, atol=1e-12)


def test_fsai_pivot_guard_and_errors(oracle):
    # tests/test_fsai.py:68-70, :116-122, :172-179
    a = np.array([[1.0, 1.0 - 1e-14], [1.0 - 1e-14, 1.0]])
    g, _, truncated = oracle.fsai(oracle.CSR.from_scipy(a), pivot_floor=1e-12)
    assert truncated == 1
    d = g.to_scipy().toarray()
    assert np.isfinite(d).all() and np.linalg.eigvalsh(d.T @ d).min() > 0
    a3 = np.array([[1.0, 1.0 - 1e-14, 0.0], [1.0 - 1e-14, 1.0, 0.0], [0.0, 0.0, 2.0]])
    for width in (2, 1):
        g, _, truncated = oracle.fsai(oracle.CSR.from_scipy(a3), width=width, step=6)
        np.testing.assert_allclose(g.to_scipy().toarray(), np.diag(1 / np.sqrt(np.diag(a3))))
    with pytest.raises(ValueError, match="positive diagonals"):
        oracle.fsai(oracle.CSR(np.array([0, 1, 1], np.int32), np.array([0], np.int32),
                               np.array([1.0])))


def test_fsai_width_one_on_blocks(oracle):
    # tests/test_fsai.py:54-59: width 1 gives I / sqrt(a_ii).
    a = np.diag(np.full(12, 3.0)) + np.diag(np.full(11, -1.0), 1) + np.diag(np.full(11, -1.0), -1)
    g, _, _ = oracle.fsai(scalar_from_blocks(oracle, a, 3), width=1)
    np.testing.assert_allclose(g.to_scipy().toarray(), np.eye(12) / np.sqrt(3))


def test_ilu0_sequential_recurrence(oracle, golden):
    # tests/test_indefinite.py:148-177
    data = golden("ilu0_recurrence.npz")
    bsr = ss.bsr_matrix(ss.csr_matrix(data["a"]), blocksize=(2, 2))
    bsr.sort_indices()
    n = 9
    factors, inverse, bad = oracle.bilu0_setup(n, 2, bsr.indptr, bsr.indices, bsr.data,
                                               factor_sweeps=2 * n + 2)
    assert bad == 0
    keys = list(zip(data["rows"], data["cols"]))
    lookup = {k: v for k, v in zip(keys, data["factors"])}
    for i in range(n):
        for e in range(bsr.indptr[i], bsr.indptr[i + 1]):
            np.testing.assert_allclose(factors[e], lookup[(i, bsr.indices[e])], rtol=1e-12,
                                       atol=1e-12)
    # Fixed-sweep apply is linear (tests/test_indefinite.py:179-192).
    rng = np.random.default_rng(83)
    x, y = rng.normal(size=(2, n * 2))

    def apply(v):
        return oracle.bilu0_apply(n, 2, bsr.indptr, bsr.indices, factors, inverse, 3, v,
                                  np.zeros_like(v), 1.0, 0.0)

    np.testing.assert_allclose(apply(0.3 * x + 0.7 * y), 0.3 * apply(x) + 0.7 * apply(y),
                               rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("size", [1, 2, 3, 4])
def test_ilu0_with_enough_sweeps_is_exact(oracle, size):
    # tests/test_indefinite.py:12-40
    rng = np.random.default_rng(61)
    n = 5
    blocks = rng.normal(size=(n, n, size, size)) * 0.03
    for i in range(n):
        blocks[i, i] = np.diag(np.arange(1, size + 1) * np.where(np.arange(size) % 2, -1.0, 1.0))
    a = blocks.transpose(0, 2, 1, 3).reshape(n * size, n * size)
    bsr = ss.bsr_matrix(a, blocksize=(size, size))
    bsr.sort_indices()
    factors, inverse, bad = oracle.bilu0_setup(n, size, bsr.indptr, bsr.indices, bsr.data,
                                               factor_sweeps=2 * n + 2)
    assert bad == 0
    x = rng.normal(size=n * size)
    y = rng.normal(size=n * size)
    z = oracle.bilu0_apply(n, size, bsr.indptr, bsr.indices, factors, inverse, n, x, y, 0.7, -0.2)
    np.testing.assert_allclose(z, 0.7 * np.linalg.solve(a, x) - 0.2 * y, rtol=1e-12, atol=1e-12)
    inv, bad = oracle.block_diag_inverse(n, size, bsr.indptr, bsr.indices, bsr.data)
    assert bad == 0
    w = oracle.block_jacobi_apply(inv, x, y, 1.0, 0.0)
    target = np.concatenate([np.linalg.solve(blocks[i, i], x[i * size:(i + 1) * size])
                             for i in range(n)])
    np.testing.assert_allclose(w, target, rtol=1e-12, atol=1e-12)


def test_bad_block_pivot(oracle):
    # tests/test_indefinite.py:142-145
    bsr = ss.bsr_matrix(np.diag([1.0, 0.0]), blocksize=(2, 2))
    _, bad = oracle.block_diag_inverse(1, 2, bsr.indptr, bsr.indices, bsr.data)
    assert bad > 0


@pytest.mark.parametrize("w", [0.0, 0.15])
def test_sqlap_reduced_operator_and_rhs(oracle, golden, w):
    # tests/test_squared_laplacian.py:12-63
    d = golden("sqlap.npz")
    lap = oracle.CSR.from_scipy(d["lap"])
    rng = np.random.default_rng(5)
    x, y = rng.normal(size=(2, len(d["free"])))
    z = oracle.sqlap_apply(lap, d["mass"], d["free"], w, x, y, 0.7, -0.2)
    np.testing.assert_allclose(z, 0.7 * d[f"reduced_w{w}"] @ x - 0.2 * y, rtol=1e-12, atol=1e-12)
    rhs = oracle.sqlap_apply(lap, d["mass"], d["free"], 0.0, d[f"bc_w{w}"],
                             np.zeros(len(d["free"])), -1.0, 0.0, boundary=True)
    np.testing.assert_allclose(rhs, d[f"rhs_w{w}"], rtol=1e-12, atol=1e-12)


def test_block_jacobi_spectrum(oracle, golden):
    # tests/test_block_challenge.py:47-60: spectrum of D^-1 (K (x) C).
    from warp_preconditioners_gb300 import problems

    bsr, _ = problems.kron_coupling(2, 1e6, seed=3)
    bsr.sort_indices()
    inv, bad = oracle.block_diag_inverse(8, 3, bsr.indptr, bsr.indices, bsr.data, tol=1e-15)
    assert bad == 0
    import scipy.linalg as sl

    p = sl.block_diag(*inv)
    eig = np.sort(np.linalg.eigvals(p @ bsr.toarray()).real)
    np.testing.assert_allclose(eig, golden("block_jacobi_spectrum.npz")["expected"], atol=1e-6)


@pytest.mark.parametrize("method", ["cg", "cr"])
def test_krylov_oracle_solves(oracle, method):
    from warp_preconditioners_gb300 import problems

    a = problems.laplacian_2d(16)
    csr = oracle.CSR.from_scipy(a)
    g, gt, _ = oracle.fsai(csr, width=8)
    b = problems.uniform_rhs(a.shape[0], 0)
    x, it, rr, atol_sq = oracle.krylov(method, oracle.Operator.csr(csr), b,
                                       M=oracle.Operator.fsai(g, gt), tol=1e-10)
    assert rr <= atol_sq and it > 0
    assert np.linalg.norm(b - a @ x) <= 1e-9 * np.linalg.norm(b)


def test_block_fsai_principal_inverse(oracle):
    # tests/test_fsai_candidates.py:15-52 (blocks = 4 gives A^-1).
    rng = np.random.default_rng(712)
    bs = 3
    n = 4 * bs
    r = rng.normal(size=(n, n))
    a = r @ r.T + np.eye(n)
    s = np.geomspace(0.01, 100, n)
    a *= s[:, None] * s[None, :]
    bsr = ss.bsr_matrix(a, blocksize=(bs, bs))
    bsr.sort_indices()
    for blocks in (1, 2, 4):
        cols, vals, _, bad = oracle.block_fsai_setup(4, bs, blocks, bsr.indptr, bsr.indices,
                                                     bsr.data)
        assert bad == 0
        g = oracle.fsai_pack(n, bs * blocks, cols, vals).to_scipy().toarray()
        for i in range(4):
            row = g[bs * i:bs * (i + 1)]
            support = np.flatnonzero(np.any(row != 0, axis=0))
            rhs = np.zeros((len(support), bs))
            rhs[-bs:, :] = np.eye(bs)
            z = np.linalg.solve(a[np.ix_(support, support)], rhs)
            expected = np.linalg.solve(np.linalg.cholesky(z[-bs:, :]), z.T)
            np.testing.assert_allclose(row[:, support], expected, rtol=2e-11, atol=1e-10)
        if blocks == 4:
            np.testing.assert_allclose(g.T @ g, np.linalg.inv(a), rtol=2e-11, atol=1e-10)


def test_fsai_setup_flop_count():
    # The counted setup is the same computation: identical factor, and the
    # count follows the operation tally of fsai.py:44-176 (width 1: one
    # reciprocal square root per row for the scale, then sqrt(z0) and
    # (z / norm) * s for the single entry = 5 operations per row).
    import scipy.sparse as ss

    from oracle import oracle

    a = ss.random(300, 300, density=0.03, random_state=np.random.default_rng(2), format="csr")
    a = (a + a.T + ss.eye(300) * 8).tocsr()
    a.sort_indices()
    c = oracle.CSR.from_scipy(a)
    f1, _, _ = oracle.fsai_setup_flops(c, width=1)
    assert f1 == 5 * 300
    counts = []
    for width in [2, 4, 8]:
        flops, cols, vals = oracle.fsai_setup_flops(c, width=width, step=1, tol=0.0)
        ref_cols, ref_vals, _, _ = oracle.fsai_setup(c, width=width, step=1, tol=0.0)
        np.testing.assert_array_equal(cols, ref_cols)
        np.testing.assert_array_equal(vals, ref_vals)
        counts.append(flops)
    assert counts[0] < counts[1] < counts[2]
