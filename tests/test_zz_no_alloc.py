"""The allocation-free FSAI apply entry point against the ordinary one.

gbpc_fsai_apply_noalloc serves callers that may not allocate device memory:
it keeps the intermediate G x in a fixed array inside libgbpc.so instead of
a cudaMalloc'd buffer.  This file is collected last so that, if it fails, a
run that stops at the first failure has already run every other test.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _entry():
    from warp_preconditioners_gb300 import _lib

    lib = _lib.load()
    fn = lib.gbpc_fsai_apply_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 6 + [ctypes.c_int] + [ctypes.c_void_p] * 3 \
        + [ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
    lib.gbpc_fsai_apply_noalloc_max_rows.restype = ctypes.c_int
    return lib, fn


def _call(fn, pre, x, y, z, alpha, beta):
    from warp_preconditioners_gb300 import _lib

    g, gt = pre.G, pre.GT
    return fn(g.nrow, _lib.ptr(g.offsets), _lib.ptr(g.columns), _lib.ptr(g.values),
              _lib.ptr(gt.offsets), _lib.ptr(gt.columns), _lib.ptr(gt.values),
              _lib.dtype_code(g.scalar_type), _lib.ptr(x), _lib.ptr(y), _lib.ptr(z),
              alpha, beta, _lib.stream(x.device))


@pytest.mark.parametrize("factor_dtype", [torch.float64, torch.float32])
def test_noalloc_apply_matches_allocating_apply(factor_dtype):
    from warp_preconditioners_gb300 import FSAI, from_scipy, problems

    dev = torch.device("cuda:0")
    a = problems.laplacian_2d(48)
    pre = FSAI(from_scipy(a, dev), max_row_size=8, factor_dtype=factor_dtype)
    _, fn = _entry()
    rng = np.random.default_rng(11)
    n = a.shape[0]
    for call in range(2):  # two calls in a row share the scratch array
        x = torch.as_tensor(rng.normal(size=n), device=dev)
        y = torch.as_tensor(rng.normal(size=n), device=dev)
        z_ref = torch.empty_like(x)
        z_new = torch.full_like(x, float("nan"))
        alpha, beta = (0.7, -0.3) if call == 0 else (1.0, 0.0)
        pre.matvec(x, y, z_ref, alpha, beta)
        assert _call(fn, pre, x, y, z_new, alpha, beta) == 0
        torch.cuda.synchronize()
        np.testing.assert_allclose(z_new.cpu().numpy(), z_ref.cpu().numpy(), rtol=1e-12,
                                   atol=1e-12)


def test_noalloc_rejects_oversize_and_keeps_working():
    from warp_preconditioners_gb300 import FSAI, _lib, from_scipy, problems

    lib, fn = _entry()
    limit = lib.gbpc_fsai_apply_noalloc_max_rows()
    assert limit == 524288
    dummy = ctypes.c_void_p(8)  # rejected before any device access
    rc = fn(limit + 1, dummy, dummy, dummy, dummy, dummy, dummy, _lib.GBPC_F64, dummy, dummy,
            dummy, 1.0, 0.0, None)
    assert rc == _lib.ERR_ARG
    assert "exceeds the fixed scratch" in _lib.last_error()
    dev = torch.device("cuda:0")
    a = problems.laplacian_2d(16)
    pre = FSAI(from_scipy(a, dev), max_row_size=4)
    x = torch.ones(a.shape[0], dtype=torch.float64, device=dev)
    z = torch.empty_like(x)
    assert _call(fn, pre, x, x, z, 1.0, 0.0) == 0
    g = pre.G.dense()
    np.testing.assert_allclose(z.cpu().numpy(), g.T @ (g @ np.ones(a.shape[0])), rtol=1e-12)
