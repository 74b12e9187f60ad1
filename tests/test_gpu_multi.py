"""Many independent systems of uneven size in one solve (MultiSystemSolver).

Five biharmonic smoothing systems on tet cubes of different sizes are
concatenated into one block-diagonal factored operator and one FSAI of the
block-diagonal Q.  Checked: that FSAI equals the per-system factors bit for
bit; every system's iteration count and backward error against the
oracle's textbook PCG of that system alone; each system's x and iteration
count identical bit for bit when it is solved by itself; a zero right-hand
side (converged at the start) and a maxiter cap that stop one system while
the others go on; the host-stepped loop equal to the graph.
"""

import numpy as np
import pytest
import torch

from gpu_helpers import cuda, host_csr, vec

pytestmark = pytest.mark.gpu

SIDES = [5, 9, 7, 12, 6]
ALPHA = 1e-4


def _berr(Q, b, x):
    return float(np.max(np.abs(b - Q @ x) / (abs(Q) @ np.abs(x) + np.abs(b))))


@pytest.fixture(scope="module")
def systems():
    from warp_preconditioners_gb300 import problems

    out = []
    for side in SIDES:
        verts, _, K, mass = problems.tet_cube(side)
        Q = problems.biharmonic(K, mass, ALPHA)
        b = problems.smoothing_rhs(verts, mass, ALPHA)[0]
        out.append((K, mass, Q, b))
    return out


def _build(parts):
    from warp_preconditioners_gb300 import FSAI, SquaredLaplacianOperator, from_scipy
    from warp_preconditioners_gb300.multi import MultiSystemSolver
    from warp_preconditioners_gb300.sparse import block_diag

    dev = cuda()
    K = block_diag([from_scipy(p[0], dev) for p in parts])
    Q = block_diag([from_scipy(p[2], dev) for p in parts])
    mass = vec(np.concatenate([p[1] for p in parts]))
    n = K.nrow
    op = SquaredLaplacianOperator(K, mass, torch.arange(n, dtype=torch.int32, device=dev),
                                  mass_weight=ALPHA)
    pre = FSAI(Q, max_row_size=8)
    sizes = [p[0].shape[0] for p in parts]
    return op, pre, sizes, MultiSystemSolver(op, pre, sizes)


def test_block_diagonal_fsai_is_the_per_system_factors(systems):
    from warp_preconditioners_gb300 import FSAI, from_scipy

    _, pre, sizes, _ = _build(systems)
    off, col, val = host_csr(pre.G)
    start = 0
    for (K, mass, Q, b), n in zip(systems, sizes):
        g = FSAI(from_scipy(Q, cuda()), max_row_size=8).G
        go, gc, gv = host_csr(g)
        lo, hi = off[start], off[start + n]
        np.testing.assert_array_equal(off[start:start + n + 1] - lo, go)
        np.testing.assert_array_equal(col[lo:hi] - start, gc)
        np.testing.assert_array_equal(val[lo:hi].view(np.int64), gv.view(np.int64))
        start += n


def test_matches_oracle_and_solo_solves(oracle, systems):
    op, pre, sizes, solver = _build(systems)
    b = vec(np.concatenate([p[3] for p in systems]))
    x = torch.zeros_like(b)
    nit, rr, atol_sq = solver.run(b, x, tol=1e-8, maxiter=20000)
    nit = nit.cpu().numpy()
    assert (rr <= atol_sq).all()
    xs = x.cpu().numpy()
    start = 0
    for s, ((K, mass, Q, bs), n) in enumerate(zip(systems, sizes)):
        qc = oracle.CSR(Q.indptr, Q.indices, Q.data)
        g, gt, _ = oracle.fsai(qc, width=8)
        kc = oracle.CSR(K.indptr, K.indices, K.data)
        x_or, it_or, _, _ = oracle.krylov("cg", oracle.Operator.sqlap(kc, mass, ALPHA), bs,
                                          M=oracle.Operator.fsai(g, gt), tol=1e-8, maxiter=20000)
        assert abs(int(nit[s]) - it_or) <= max(2, int(0.02 * it_or)), (s, nit[s], it_or)
        xi = xs[start:start + n]
        assert _berr(Q, bs, xi) <= max(4 * _berr(Q, bs, x_or), 1e-14), s
        # the same system alone: identical iterates
        _, _, _, alone = _build([systems[s]])
        xa = torch.zeros(n, dtype=torch.float64, device=cuda())
        nit_a, _, _ = alone.run(vec(bs), xa, tol=1e-8, maxiter=20000)
        assert int(nit_a.item()) == int(nit[s])
        np.testing.assert_array_equal(xa.cpu().numpy().view(np.int64), xi.view(np.int64))
        start += n
    # repeated run of the captured graph, and the host-stepped loop
    x2 = torch.zeros_like(b)
    solver.run(b, x2, tol=1e-8, maxiter=20000)
    assert torch.equal(x, x2)
    from warp_preconditioners_gb300.multi import MultiSystemSolver

    host = MultiSystemSolver(op, pre, sizes, use_cuda_graph=False)
    x3 = torch.zeros_like(b)
    nit3, _, _ = host.run(b, x3, tol=1e-8, maxiter=20000)
    assert torch.equal(x, x3) and np.array_equal(nit3.cpu().numpy(), nit)


def test_converged_and_capped_systems_stop_alone(systems):
    _, _, sizes, solver = _build(systems)
    parts = [p[3].copy() for p in systems]
    parts[1][:] = 0.0  # converged at the start
    b = vec(np.concatenate(parts))
    x = torch.zeros_like(b)
    nit, rr, atol_sq = solver.run(b, x, tol=1e-8, maxiter=20000)
    nit = nit.cpu().numpy()
    assert nit[1] == 0
    s1 = slice(sum(sizes[:1]), sum(sizes[:2]))
    assert torch.count_nonzero(x[s1]) == 0
    assert (nit[[0, 2, 3, 4]] > 0).all()
    # cap: every system stops at 5 iterations
    x.zero_()
    nit5, rr5, atol5 = solver.run(b, x, tol=1e-12, maxiter=5)
    nit5 = nit5.cpu().numpy()
    assert nit5[1] == 0 and (nit5[[0, 2, 3, 4]] == 5).all()
    with pytest.raises(ValueError):
        from warp_preconditioners_gb300.multi import MultiSystemSolver

        MultiSystemSolver(solver.A, solver.M, sizes[:-1])


def test_cluster_solver_matches_each_system_alone(oracle, systems):
    # One launch, one thread-block cluster per system, each system with its
    # own operators: biharmonic factored operators with FSAI, a Laplacian
    # with FSAI, a Laplacian with no preconditioner, and a zero right-hand
    # side.  Each system's x and iteration count equal the drop-in solver's
    # on that system alone (the same cluster kernel below 32,768 rows).
    from warp_preconditioners_gb300 import (FSAI, SparseOperator, SquaredLaplacianOperator,
                                            from_scipy, linear, problems)
    from warp_preconditioners_gb300.multi import ClusterSolver

    dev = cuda()
    pairs, rhs, mats = [], [], []
    for K, mass, Q, b in systems:
        n = K.shape[0]
        op = SquaredLaplacianOperator(from_scipy(K, dev), vec(mass),
                                      torch.arange(n, dtype=torch.int32, device=dev),
                                      mass_weight=ALPHA)
        pairs.append((op, FSAI(from_scipy(Q, dev), max_row_size=8)))
        rhs.append(b)
        mats.append(Q)
    for side, pre in ((40, True), (30, False)):
        a = problems.laplacian_2d(side)
        A = from_scipy(a, dev)
        pairs.append((SparseOperator(A), FSAI(A, max_row_size=8) if pre else None))
        rhs.append(problems.uniform_rhs(a.shape[0], side))
        mats.append(a)
    rhs[1] = np.zeros_like(rhs[1])
    solver = ClusterSolver(pairs)
    assert solver.cluster_size in (8, 16)
    bs = [vec(b) for b in rhs]
    xs = [torch.zeros_like(b) for b in bs]
    nit, rr, atol_sq = solver.run(bs, xs, tol=1e-8, maxiter=20000)
    nit = nit.cpu().numpy()
    assert nit[1] == 0 and torch.count_nonzero(xs[1]) == 0
    assert (rr <= atol_sq).all()
    for s, ((A, M), b, x) in enumerate(zip(pairs, bs, xs)):
        alone = torch.zeros_like(b)
        it, _, _ = linear.Solver("cg", A, M).run(b, alone, tol=1e-8, maxiter=20000)
        assert int(it.item()) == int(nit[s]), s
        assert torch.equal(alone, x), s
    # a second run gives the same bits
    xs2 = [torch.zeros_like(b) for b in bs]
    solver.run(bs, xs2, tol=1e-8, maxiter=20000)
    assert all(torch.equal(a, b) for a, b in zip(xs, xs2))
    # against the oracle's PCG on the first biharmonic system
    K, mass, Q, b0 = systems[0]
    qc = oracle.CSR(Q.indptr, Q.indices, Q.data)
    g, gt, _ = oracle.fsai(qc, width=8)
    kc = oracle.CSR(K.indptr, K.indices, K.data)
    _, it_or, _, _ = oracle.krylov("cg", oracle.Operator.sqlap(kc, mass, ALPHA), b0,
                                   M=oracle.Operator.fsai(g, gt), tol=1e-8, maxiter=20000)
    assert abs(int(nit[0]) - it_or) <= max(2, int(0.02 * it_or))
