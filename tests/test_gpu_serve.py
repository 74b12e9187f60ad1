"""Serving loop on the GPU: a request gives bit-identical x alone and in
the mix; returned solutions meet the residual tolerance; resident systems
stay within their byte estimate and release everything on eviction."""

import numpy as np
import pytest
import scipy.sparse as ss
import torch

from warp_preconditioners_gb300 import _lib, serve

pytestmark = pytest.mark.gpu

TOL = 1e-8


def small_stream():
    rng = np.random.default_rng(5)
    out = []
    for i in range(18):
        kind = serve.KINDS[i % 2]
        side = int(rng.integers(5, 10)) if kind == "laplacian" else int(rng.integers(4, 8))
        out.append(serve.Request(i, kind, side, int(rng.integers(1, 9)), 0.0005 * i,
                                 int(rng.integers(0, 2**31 - 1))))
    return out


@pytest.fixture(scope="module")
def catalog():
    cat = serve.Catalog()
    cat.prebuild({r.key for r in small_stream()}, threads=4)
    return cat


def host_matrix(h):
    return h.assembled()  # L, or the assembled alpha M + K M^-1 K


@pytest.mark.parametrize("cluster_rhs", [False, True])
def test_alone_equals_mixed(catalog, cluster_rhs):
    stream = small_stream()
    mixed_ex = serve.GpuExecutor(catalog, slots=6, tol=TOL, cluster_rhs=cluster_rhs)
    mixed = serve.Server(mixed_ex).run(stream)
    assert all(r.ok for r in mixed), [r.error for r in mixed if not r.ok]
    # Each request again, alone, on a fresh executor (fresh systems and slots).
    alone_ex = serve.GpuExecutor(catalog, slots=1, tol=TOL, cluster_rhs=cluster_rhs)
    for req, m in zip(stream, mixed):
        a = serve.Server(alone_ex).run([serve.Request(req.rid, req.kind, req.side, req.k, 0.0,
                                                      req.seed)])[0]
        assert a.ok
        assert a.iterations == m.iterations, req
        assert torch.equal(a.x, m.x), req


def test_solutions_meet_tolerance_and_match_sequential(catalog):
    stream = small_stream()
    served = serve.Server(serve.GpuExecutor(catalog, slots=4, tol=TOL)).run(stream)
    seq = serve.Server(serve.GpuExecutor(catalog, sequential=True, tol=TOL)).run(stream)
    for req, r, s in zip(stream, served, seq):
        assert r.ok and s.ok
        A = host_matrix(catalog.get(req.key))
        b = serve.request_rhs(req).numpy()
        x = r.x.numpy()
        res = np.linalg.norm(b - A @ x, axis=0) / np.linalg.norm(b, axis=0)
        assert res.max() < 50 * TOL, (req, res)
        # batched and single-vector recurrences agree to the solve tolerance
        xs = s.x.numpy()
        assert np.abs(x - xs).max() <= 1e-6 * np.abs(xs).max(), req
        assert all(abs(a - b) <= 2 for a, b in zip(r.iterations, s.iterations)), req


def test_resident_bytes_within_estimate_and_released(catalog):
    import gc

    ex = serve.GpuExecutor(catalog, slots=2, tol=TOL)
    gc.collect()  # objects of earlier tests release their memory now, not below
    torch.cuda.synchronize()
    live0 = _lib.live_device_bytes()
    srv = serve.Server(ex, budget_bytes=4 << 30)
    keys = [("biharmonic", 7), ("laplacian", 9)]
    srv.prepare(keys)
    for key in keys:
        nbytes = srv.resident[key][1]
        assert 0 < nbytes <= ex.estimate(key), (key, nbytes, ex.estimate(key))
    assert srv.used == sum(v[1] for v in srv.resident.values())
    assert _lib.live_device_bytes() > live0
    # Evict everything: the library's live bytes return to where they were.
    srv.budget = 0
    srv._make_room(0)
    gc.collect()
    torch.cuda.synchronize()
    assert not srv.resident and srv.used == 0
    assert _lib.live_device_bytes() == live0


def test_tight_budget_still_serves_everything(catalog):
    stream = small_stream()
    ex = serve.GpuExecutor(catalog, slots=3, tol=TOL)
    # Room for the largest estimate and little more: systems must be evicted.
    biggest = max(ex.estimate(r.key) for r in stream)
    srv = serve.Server(ex, budget_bytes=int(1.1 * biggest))
    out = srv.run(stream)
    assert all(r.ok for r in out), [r.error for r in out if not r.ok]
    assert srv.stats["evictions"] > 0
    assert srv.peak <= srv.budget


def test_merged_requests_match_alone_within_tolerance(catalog):
    # Requests queued for one system are merged into one batched solve
    # (merge_rhs): each keeps its own CG recurrence, so its x equals the
    # unmerged solve to the solve tolerance (the fold of the batched dot
    # products depends on the group's width, so not bit for bit).
    keys = [("laplacian", 7), ("biharmonic", 5)]
    for key in keys:
        catalog.get(key)
    stream = [serve.Request(i, *keys[i % 2], 1 + i % 3, 0.0, 1000 + i) for i in range(8)]
    merged_ex = serve.GpuExecutor(catalog, slots=2, tol=TOL, merge_rhs=16)
    merged = serve.Server(merged_ex).run(stream)
    alone_ex = serve.GpuExecutor(catalog, slots=1, tol=TOL)
    alone = serve.Server(alone_ex).run(stream)
    for req, m, a in zip(stream, merged, alone):
        assert m.ok and a.ok, (m.error, a.error)
        x, xa = m.x.numpy(), a.x.numpy()
        assert x.shape == xa.shape == (req.n, req.k)
        assert np.abs(x - xa).max() <= 1e-6 * np.abs(xa).max(), req
        assert all(abs(i - j) <= max(2, 0.03 * j) for i, j in zip(m.iterations, a.iterations))
        A = host_matrix(catalog.get(req.key))
        b = serve.request_rhs(req).numpy()
        res = np.linalg.norm(b - A @ x, axis=0) / np.linalg.norm(b, axis=0)
        assert res.max() < 50 * TOL, (req, res)


def test_wide_factors_for_large_systems_meet_tolerance(catalog):
    # Systems at or above wide_from get a width-48 factor (grown two entries
    # a step); every request still meets the solve tolerance.
    stream = small_stream()
    ex = serve.GpuExecutor(catalog, slots=4, tol=TOL, wide_from=1)
    assert all(ex.width_for(catalog.get(r.key)) == 48 for r in stream)
    served = serve.Server(ex).run(stream)
    for req, r in zip(stream, served):
        assert r.ok, r.error
        A = host_matrix(catalog.get(req.key))
        b = serve.request_rhs(req).numpy()
        res = np.linalg.norm(b - A @ r.x.numpy(), axis=0) / np.linalg.norm(b, axis=0)
        assert res.max() < 50 * TOL, (req, res)
