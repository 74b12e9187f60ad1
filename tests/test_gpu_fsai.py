"""FSAI on the GPU against the oracle (bit-exact supports and values) and the
reference's known answers.  Mirrors tests/test_fsai.py of the reference."""

import numpy as np
import pytest
import scipy.sparse as ss
import torch

from gpu_helpers import cuda, host_csr, oracle_csr, to_bsr, vec

pytestmark = pytest.mark.gpu


def assert_same_factor(g_gpu, g_oracle):
    off, col, val = host_csr(g_gpu)
    np.testing.assert_array_equal(off, g_oracle.offsets)
    np.testing.assert_array_equal(col, g_oracle.columns)
    # Bit-exact: same operations in the same order without contraction.
    np.testing.assert_array_equal(val, g_oracle.values)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("step", [1, 3])
@pytest.mark.parametrize("tol", [0.0, 0.003, 0.1])
def test_greedy_support_matches_oracle_and_golden(golden, oracle, dtype, step, tol):
    from warp_preconditioners_gb300 import FSAI

    data = golden("fsai_greedy.npz")
    a = data["a"]
    npdt = np.float64 if dtype == torch.float64 else np.float32
    raw = to_bsr(a, dtype, block=3)
    pre = FSAI(raw, max_row_size=8, kap_tolerance=tol, max_step_size=step)
    g_or, gt_or, _ = oracle.fsai(oracle_csr(oracle, a, npdt, block=3), width=8, step=step,
                                 tol=tol)
    assert_same_factor(pre.G, g_or)
    assert_same_factor(pre.GT, gt_or)
    expected = data[f"g_tol{tol}_step{step}"]
    rtol, atol = (3e-5, 1e-6) if dtype == torch.float32 else (1e-10, 1e-13)
    np.testing.assert_allclose(pre.G.dense(), expected, rtol=rtol, atol=atol)


@pytest.mark.parametrize("step", [1, 3])
def test_full_pattern_apply_aliases(golden, step):
    from warp_preconditioners_gb300 import FSAI

    d = golden("fsai_full.npz")
    pre = FSAI(to_bsr(d["a8"]), max_row_size=8, kap_tolerance=0, max_step_size=step)
    g = pre.G.dense()
    np.testing.assert_allclose(g.T @ g, d["inv8"], rtol=1e-10, atol=1e-12)
    assert np.allclose(g, np.tril(g))
    x = vec(d["x8"])
    y = vec(d["y8"])
    expected = 1.7 * g.T @ g @ d["x8"] - 0.3 * d["y8"]
    pre.matvec(x, y, y, 1.7, -0.3)
    np.testing.assert_allclose(y.cpu().numpy(), expected, rtol=1e-12, atol=1e-12)


def test_scaled_supports_aliases_nan_and_graph(golden, oracle):
    from warp_preconditioners_gb300 import FSAI

    a = golden("fsai_scaled.npz")["a"]
    pre = FSAI(to_bsr(a), max_row_size=5, kap_tolerance=0)
    g_or, _, _ = oracle.fsai(oracle_csr(oracle, a), width=5, tol=0.0)
    assert_same_factor(pre.G, g_or)
    g = pre.G.dense()
    rng = np.random.default_rng(18)
    for alias in ["none", "xz", "yz", "xy", "xyz"]:
        x = vec(rng.normal(size=20))
        y = x if alias in ["xy", "xyz"] else vec(rng.normal(size=20))
        z = x if alias in ["xz", "xyz"] else y if alias == "yz" else torch.empty_like(x)
        expected = 0.7 * g.T @ g @ x.cpu().numpy() - 1.2 * y.cpu().numpy()
        pre.matvec(x, y, z, 0.7, -1.2)
        np.testing.assert_allclose(z.cpu().numpy(), expected, rtol=1e-12, atol=1e-10)
    # NaN in y must not leak when beta == 0.
    x = vec(rng.normal(size=20))
    y = torch.full_like(x, float("nan"))
    pre.matvec(x, y, y, 1.0, 0.0)
    assert torch.isfinite(y).all()
    # Graph capture and replay of the apply.
    z = torch.empty_like(x)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        pre.matvec(x, y, z, 1.0, 0.0)
    torch.cuda.current_stream().wait_stream(s)
    graph = torch.cuda.CUDAGraph()
    z.zero_()
    with torch.cuda.graph(graph):
        pre.matvec(x, y, z, 1.0, 0.0)
    z.zero_()
    graph.replay()
    torch.cuda.synchronize()
    np.testing.assert_allclose(z.cpu().numpy(), g.T @ g @ x.cpu().numpy(), rtol=1e-12, atol=1e-10)


def test_pivot_guard_and_validation():
    from warp_preconditioners_gb300 import FSAI

    a = np.array([[1.0, 1.0 - 1e-14], [1.0 - 1e-14, 1.0]])
    m = FSAI(to_bsr(a), pivot_floor=1e-12)
    assert m.truncated_rows == 1
    g = m.G.dense()
    assert np.isfinite(g).all() and np.linalg.eigvalsh(g.T @ g).min() > 0
    a3 = np.array([[1.0, 1.0 - 1e-14, 0.0], [1.0 - 1e-14, 1.0, 0.0], [0.0, 0.0, 2.0]])
    pre = FSAI(to_bsr(a3), max_row_size=2, max_step_size=6)
    assert pre.truncated_rows == 1
    np.testing.assert_allclose(pre.G.dense(), np.diag(1 / np.sqrt(np.diag(a3))))
    pre = FSAI(to_bsr(a3), max_row_size=1, max_step_size=6)
    np.testing.assert_allclose(pre.G.dense(), np.diag(1 / np.sqrt(np.diag(a3))))
    with pytest.raises(ValueError, match="positive diagonals"):
        FSAI(to_bsr(np.diag([1.0, -1.0])))
    for value in [0, -1, 65, 1.5]:
        with pytest.raises(ValueError, match="max_step_size"):
            FSAI(to_bsr(np.eye(3)), max_step_size=value)
    with pytest.raises(ValueError, match="apply_lanes"):
        FSAI(to_bsr(np.eye(4)), apply_lanes=3)
    with pytest.raises(ValueError, match="positive diagonal"):
        FSAI(to_bsr(np.eye(3) * 1e100), factor_dtype=torch.float32)


@pytest.mark.parametrize("step", [2, 3])
def test_path_graph_counts_and_values(golden, step):
    from warp_preconditioners_gb300 import FSAI

    d = golden("fsai_path.npz")
    pre = FSAI(to_bsr(d["a"]), max_row_size=8, max_step_size=step, kap_tolerance=0.0)
    np.testing.assert_array_equal(np.diff(pre.G.offsets.cpu().numpy()), d["counts"])
    np.testing.assert_allclose(pre.G.dense(), d["g"], rtol=1e-12, atol=1e-15)


def test_zero_tolerance_full_width(golden):
    from warp_preconditioners_gb300 import FSAI

    d = golden("fsai_full.npz")
    pre = FSAI(to_bsr(d["a32"]), max_row_size=32, kap_tolerance=0, max_step_size=3)
    np.testing.assert_array_equal(np.diff(pre.G.offsets.cpu().numpy()), np.arange(1, 33))
    g = pre.G.dense()
    np.testing.assert_allclose(g.T @ g, d["inv32"], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("width,step", [(1, 1), (2, 1), (3, 5), (8, 1), (8, 2), (12, 2),
                                        (16, 1), (16, 3), (48, 1), (48, 2), (64, 3), (64, 64)])
def test_biharmonic_tet_cube_bit_exact(oracle, width, step):
    # The assembled smoothing operator of the benchmark, on a small cube:
    # 65-entry rows, exact ties, numerically nonsymmetric SpGEMM values.
    from warp_preconditioners_gb300 import FSAI, problems

    _, _, K, mass = problems.tet_cube(9)
    q = problems.biharmonic(K, mass, 1e-4)
    pre = FSAI(to_bsr(q), max_row_size=width, max_step_size=step, kap_tolerance=1e-3)
    g_or, gt_or, trunc = oracle.fsai(oracle_csr(oracle, q), width=width, step=step, tol=1e-3)
    assert pre.truncated_rows == trunc
    assert_same_factor(pre.G, g_or)
    assert_same_factor(pre.GT, gt_or)


@pytest.mark.parametrize("width,step", [(8, 2), (16, 2)])
def test_wide_frontier_overflow_rerun_bit_exact(oracle, width, step):
    # ~290 entries per row: frontiers exceed the first pass's candidate
    # table (512 slots), so those rows are rebuilt by the rerun with a table
    # that cannot overflow.
    from warp_preconditioners_gb300 import FSAI

    rng = np.random.default_rng(83)
    n = 1500
    m = ss.random(n, n, density=0.1, random_state=rng, data_rvs=lambda k: rng.uniform(-1, 1, k))
    a = (m + m.T).tocsr()
    a = a + ss.diags(np.abs(a).sum(axis=1).A1 + 1.0)
    a.sort_indices()
    pre = FSAI(to_bsr(a), max_row_size=width, max_step_size=step, kap_tolerance=0.0)
    g_or, gt_or, trunc = oracle.fsai(oracle_csr(oracle, a), width=width, step=step, tol=0.0)
    # Some row's final support meets more distinct columns below it than the
    # first table holds, so the rerun ran.
    widest = 0
    for i in range(0, n, 7):
        sup = g_or.columns[g_or.offsets[i]:g_or.offsets[i + 1]]
        cols = np.unique(np.concatenate([a.indices[a.indptr[c]:a.indptr[c + 1]] for c in sup]))
        widest = max(widest, int((cols < i).sum()) + len(sup))
    assert widest > 512
    assert pre.truncated_rows == trunc
    assert_same_factor(pre.G, g_or)
    assert_same_factor(pre.GT, gt_or)


@pytest.mark.parametrize("factor_dtype", [torch.float32, torch.bfloat16])
def test_compressed_factor_apply(oracle, factor_dtype):
    from warp_preconditioners_gb300 import FSAI, problems

    a = problems.laplacian_2d(32)
    pre = FSAI(to_bsr(a), max_row_size=8, factor_dtype=factor_dtype)
    g64, _, _ = oracle.fsai(oracle_csr(oracle, a), width=8)
    np.testing.assert_array_equal(pre.G.offsets.cpu().numpy(), g64.offsets)
    np.testing.assert_array_equal(
        pre.G.values.cpu().to(torch.float64).numpy(),
        torch.as_tensor(g64.values).to(factor_dtype).to(torch.float64).numpy())
    np.testing.assert_array_equal(pre.GT.dense(), pre.G.dense().T)
    g = pre.G.dense()
    rng = np.random.default_rng(72)
    x = vec(rng.normal(size=a.shape[0]))
    y = vec(rng.normal(size=a.shape[0]))
    expected = 0.7 * g.T @ (g @ x.cpu().numpy()) - 0.3 * y.cpu().numpy()
    pre.matvec(x, y, x, 0.7, -0.3)
    np.testing.assert_allclose(x.cpu().numpy(), expected, rtol=1e-12, atol=1e-12)


def test_laplacian_2d_64_bit_exact(oracle):
    # The 4,096-unknown plain configuration, width 8, single-entry growth.
    from warp_preconditioners_gb300 import FSAI, problems

    a = problems.laplacian_2d(64)
    pre = FSAI(to_bsr(a), max_row_size=8)
    g_or, gt_or, _ = oracle.fsai(oracle_csr(oracle, a), width=8)
    assert_same_factor(pre.G, g_or)
    assert_same_factor(pre.GT, gt_or)


def test_empty_and_single_row():
    from warp_preconditioners_gb300 import FSAI

    pre = FSAI(to_bsr(np.array([[4.0]])))
    np.testing.assert_allclose(pre.G.dense(), [[0.5]])
    x = vec([2.0])
    z = torch.empty_like(x)
    pre.matvec(x, x, z, 1.0, 0.0)
    np.testing.assert_allclose(z.cpu().numpy(), [0.5])
