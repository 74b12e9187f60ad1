"""Fixed-support FSAI refit on the GPU: bit-exact against the oracle's
restatement of fsai_reuse.py's `refit`, and the behaviour of the reference's
tests/test_updates.py (in-place values, G^T = G.T, local solves, rollback on
invalid input, topology checks, graph replay after an update)."""

import numpy as np
import pytest
import torch

from gpu_helpers import cuda, host_csr, oracle_csr, to_bsr, vec

pytestmark = pytest.mark.gpu


def spd12(seed=48):
    r = np.random.default_rng(seed).normal(size=(12, 12))
    return r @ r.T + np.eye(12) * 3


def same_topology_copy(B, columns=None, values=None):
    from warp_preconditioners_gb300 import BsrMatrix

    return BsrMatrix(B.nrow, B.ncol, B.block_shape, B.offsets.clone(),
                     B.columns.clone() if columns is None else columns,
                     B.values.clone() if values is None else values)


@pytest.mark.parametrize("block", [1, 3])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("step", [1, 3])
def test_refit_local_solves_and_rollback(block, dtype, step):
    from warp_preconditioners_gb300 import FSAI

    a = spd12()
    A = to_bsr(a, dtype, block)
    m = FSAI(A, max_row_size=5, reuse_pattern=True, factor_dtype=torch.float32,
             max_step_size=step)
    gptr, tptr = m.G.values.data_ptr(), m.GT.values.data_ptr()
    b = a + np.diag(np.arange(12.0))
    B = to_bsr(b, dtype, block)
    assert m.update(B) is m
    assert (m.G.values.data_ptr(), m.GT.values.data_ptr()) == (gptr, tptr)
    g = m.G.dense()
    np.testing.assert_array_equal(m.GT.dense(), g.T)
    off, col, _ = host_csr(m.G)
    for i in range(12):
        support = col[off[i]:off[i + 1]]
        e = np.zeros(len(support))
        e[-1] = 1
        z = np.linalg.solve(b[np.ix_(support, support)], e)
        np.testing.assert_allclose(g[i, support], z / np.sqrt(z[-1]), rtol=2e-4, atol=2e-7)
    # The operator applies the refitted factor.
    x = vec(np.linspace(-1, 1, 12), dtype)
    y = torch.zeros_like(x)
    m.matvec(x, y, y, 1.0, 0.0)
    np.testing.assert_allclose(y.cpu().numpy(), g.T @ g @ x.cpu().numpy(), rtol=1e-5, atol=1e-6)
    # Invalid values: error, previous factor kept.
    invalid = same_topology_copy(B, values=torch.zeros_like(B.values))
    with pytest.raises(ValueError, match="positive diagonals"):
        m.update(invalid)
    np.testing.assert_array_equal(m.G.dense(), g)
    # Changed sparsity: error, previous factor kept.
    cols = B.columns.clone()
    cols[0] += 1
    with pytest.raises(ValueError, match="sparsity"):
        m.update(same_topology_copy(B, columns=cols))
    np.testing.assert_array_equal(m.G.dense(), g)
    # Same object, changed values, then a no-argument update.
    B.values.copy_(A.values)
    m.update()
    fresh = FSAI(A, max_row_size=12, kap_tolerance=0, reuse_pattern=True)
    fresh.update(B)
    np.testing.assert_allclose(fresh.G.dense().T @ fresh.G.dense(), np.linalg.inv(a),
                               rtol=2e-4, atol=1e-7)
    assert fresh.quality(probes=2) < (1e-5 if dtype == torch.float32 else 1e-12)


@pytest.mark.parametrize("mdt,fdt", [(torch.float64, torch.float64),
                                     (torch.float64, torch.float32),
                                     (torch.float32, torch.float32)])
@pytest.mark.parametrize("width,step", [(8, 1), (8, 2), (12, 2), (24, 3), (48, 1)])
def test_refit_bit_exact_against_oracle(oracle, mdt, fdt, width, step):
    from warp_preconditioners_gb300 import FSAI, problems

    _, _, K, mass = problems.tet_cube(8)
    q1 = problems.biharmonic(K, mass, 1e-4)
    q2 = problems.biharmonic(K, mass, 3e-3)  # same pattern, new values
    assert (q1.indptr == q2.indptr).all() and (q1.indices == q2.indices).all()
    npm = np.float64 if mdt == torch.float64 else np.float32
    npf = np.float64 if fdt == torch.float64 else np.float32
    pre = FSAI(to_bsr(q1, mdt), max_row_size=width, max_step_size=step, reuse_pattern=True,
               factor_dtype=fdt)
    pre.update(to_bsr(q2, mdt))
    off, col, val = host_csr(pre.G)
    g = oracle.CSR(off, col, val.astype(npf))
    expected, bd, br = oracle.fsai_refit(oracle_csr(oracle, q2, npm), g, factor_dtype=npf)
    assert bd == br == 0
    np.testing.assert_array_equal(val, expected)
    np.testing.assert_array_equal(pre.GT.dense(), pre.G.dense().T)


def test_bfloat16_factor_refit_rounds_the_float_refit(oracle):
    from warp_preconditioners_gb300 import FSAI, problems

    _, _, K, mass = problems.tet_cube(7)
    q1 = problems.biharmonic(K, mass, 1e-4)
    q2 = problems.biharmonic(K, mass, 2e-3)
    pre = FSAI(to_bsr(q1), max_row_size=8, reuse_pattern=True, factor_dtype=torch.bfloat16)
    pre.update(to_bsr(q2))
    off, col, val = host_csr(pre.G.__class__(pre.G.nrow, pre.G.ncol, (1, 1), pre.G.offsets,
                                             pre.G.columns, pre.G.values.float()))
    f32, bd, br = oracle.fsai_refit(oracle_csr(oracle, q2), oracle.CSR(off, col, val),
                                    factor_dtype=np.float32)
    assert bd == br == 0
    expected = torch.from_numpy(f32).to(torch.bfloat16).float().numpy()
    np.testing.assert_array_equal(val, expected)


def test_block_update_and_graph_replay():
    from warp_preconditioners_gb300 import BlockJacobi, FSAI

    a = np.array([[3.0, 0.4, 0], [0.4, 2, 0], [0, 0, 4.0]])
    A = to_bsr(a, block=3)
    B = to_bsr(2 * a, block=3)
    for m in [BlockJacobi(A), FSAI(A, max_row_size=3, kap_tolerance=0, reuse_pattern=True)]:
        x = vec([1.0, 2.0, 3.0])
        y = torch.zeros_like(x)
        m.matvec(x, y, y, 1.0, 0.0)
        graph = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            with torch.cuda.graph(graph, stream=s):
                m.matvec(x, y, y, 1.0, 0.0)
        torch.cuda.current_stream().wait_stream(s)
        m.update(B)
        graph.replay()
        torch.cuda.synchronize()
        np.testing.assert_allclose(y.cpu().numpy(), np.linalg.solve(2 * a, [1.0, 2.0, 3.0]),
                                   rtol=1e-12)
        B.values.zero_()
        with pytest.raises(ValueError):
            m.update(B)
        m.matvec(x, y, y, 1.0, 0.0)
        np.testing.assert_allclose(y.cpu().numpy(), np.linalg.solve(2 * a, [1.0, 2.0, 3.0]),
                                   rtol=1e-12)
        B.values.copy_(2 * A.values)


def test_numeric_zero_becomes_nonzero_inside_block():
    from warp_preconditioners_gb300 import FSAI

    a = np.array([[4.0, 1.0, 0.0], [1.0, 4.0, 1.0], [0.0, 1.0, 4.0]])
    b = a + 0.2 * np.ones((3, 3))
    A, B = to_bsr(a, block=3), to_bsr(b, block=3)
    m = FSAI(A, max_row_size=3, kap_tolerance=0, reuse_pattern=True)
    m.update(A)
    np.testing.assert_allclose(m.G.dense().T @ m.G.dense(), np.linalg.inv(a), atol=1e-13)
    m.update(B)
    np.testing.assert_allclose(m.G.dense().T @ m.G.dense(), np.linalg.inv(b), atol=1e-13)


def test_refit_requires_explicit_plan():
    from warp_preconditioners_gb300 import FSAI

    a = to_bsr(np.eye(3))
    with pytest.raises(ValueError, match="reuse_pattern=True"):
        FSAI(a).update(a)


def test_refit_signature_checks():
    from warp_preconditioners_gb300 import FSAI

    A = to_bsr(spd12())
    m = FSAI(A, max_row_size=4, reuse_pattern=True)
    with pytest.raises(ValueError, match="original shape"):
        m.update(to_bsr(spd12(), torch.float32))
    with pytest.raises(ValueError, match="original shape"):
        m.update(to_bsr(np.eye(6) * 2))
    with pytest.raises(ValueError, match="BsrMatrix"):
        m.update(np.eye(12))
    with pytest.raises(ValueError, match="probes"):
        m.quality(probes=0)


def test_empty_reusable_fsai():
    from warp_preconditioners_gb300 import BsrMatrix, FSAI

    for dtype in [torch.float32, torch.float64]:
        dev = cuda()
        matrix = BsrMatrix(0, 0, (1, 1), torch.zeros(1, dtype=torch.int32, device=dev),
                           torch.zeros(0, dtype=torch.int32, device=dev),
                           torch.zeros(0, dtype=dtype, device=dev))
        pre = FSAI(matrix, reuse_pattern=True)
        assert pre.update() is pre
        assert pre.G.nnz == 0 and pre.GT.nnz == 0
        v = torch.empty(0, dtype=dtype, device=dev)
        pre.matvec(v, v, v, 1.0, 0.0)
        torch.cuda.synchronize()


def test_build_and_refit_in_chunks(oracle, monkeypatch):
    # The build by rounds and the wide refit hold the device state of a
    # chunk of rows at a time (GBPC_FSAI_CHUNK_ROWS caps it); four chunks of
    # the 12^3 cube give the oracle's factor and refit bit for bit.
    from warp_preconditioners_gb300 import FSAI, problems

    _, _, K, mass = problems.tet_cube(12)
    q1 = problems.biharmonic(K, mass, 1e-4)
    q2 = problems.biharmonic(K, mass, 3e-3)
    monkeypatch.setenv("GBPC_FSAI_CHUNK_ROWS", "500")
    pre = FSAI(to_bsr(q1), max_row_size=24, max_step_size=2, kap_tolerance=1e-3,
               reuse_pattern=True)
    g_or, _, trunc = oracle.fsai(oracle_csr(oracle, q1), width=24, step=2, tol=1e-3)
    off, col, val = host_csr(pre.G)
    np.testing.assert_array_equal(off, g_or.offsets)
    np.testing.assert_array_equal(col, g_or.columns)
    np.testing.assert_array_equal(val, g_or.values)
    assert pre.truncated_rows == trunc
    pre.update(to_bsr(q2))
    off, col, val = host_csr(pre.G)
    expected, bd, br = oracle.fsai_refit(oracle_csr(oracle, q2), oracle.CSR(off, col, val))
    assert bd == br == 0
    np.testing.assert_array_equal(val, expected)
