"""The allocation-free FSAI apply entry point.

gbpc_fsai_apply_noalloc serves callers that may not allocate device memory
(a host that hands the library a fixed device pool, or a path that must stay
free of allocation calls): it keeps the intermediate G x in a fixed array
inside libgbpc.so instead of a cudaMalloc'd buffer.  Its results are checked
against the dense product alpha G^T G x + beta y and against the ordinary
allocating apply, on two calls in a row (every call shares the one array),
with the aliasing and NaN rules its declaration promises.  This file is
collected last so that, if it fails, a run that stops at the first failure
has already run every other test.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

RTOL = 1e-12


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
    dev = z.device
    return fn(g.nrow, _lib.ptr(g.offsets), _lib.ptr(g.columns), _lib.ptr(g.values),
              _lib.ptr(gt.offsets), _lib.ptr(gt.columns), _lib.ptr(gt.values),
              _lib.dtype_code(g.scalar_type), _lib.ptr(x), _lib.ptr(y), _lib.ptr(z),
              alpha, beta, _lib.stream(dev))


def _dense_apply(pre, x, y, alpha, beta):
    g = pre.G.dense()
    out = np.zeros(g.shape[0])
    if alpha != 0.0:
        out += alpha * (g.T @ (g @ x))
    if beta != 0.0:
        out += beta * y
    return out


def test_zero_row_first_call_reserves_scratch():
    """A call with n = 0 (and no arrays) reserves the scratch array and succeeds;
    the next real call on the device then works as usual."""
    from warp_preconditioners_gb300 import FSAI, from_scipy, problems

    lib, fn = _entry()
    dev = torch.device("cuda:0")
    torch.cuda.init()
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    rc = fn(0, None, None, None, None, None, None, 0, None, None, None, 1.0, 0.0, stream)
    assert rc == 0
    a = problems.laplacian_2d(12)
    pre = FSAI(from_scipy(a, dev), max_row_size=6)
    x = torch.as_tensor(np.linspace(-1.0, 1.0, a.shape[0]), device=dev)
    z = torch.empty_like(x)
    assert _call(fn, pre, x, None, z, 1.0, 0.0) == 0
    torch.cuda.synchronize()
    np.testing.assert_allclose(z.cpu().numpy(), _dense_apply(pre, x.cpu().numpy(), None, 1.0, 0.0),
                               rtol=RTOL, atol=1e-14)


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
        np.testing.assert_allclose(z_new.cpu().numpy(), z_ref.cpu().numpy(), rtol=RTOL,
                                   atol=1e-12)
        np.testing.assert_allclose(
            z_new.cpu().numpy(),
            _dense_apply(pre, x.cpu().numpy(), y.cpu().numpy(), alpha, beta),
            rtol=1e-11, atol=1e-11)


@pytest.mark.parametrize("case", ["z_is_x", "z_is_y", "x_is_y_is_z", "nan_y_beta0",
                                  "alpha0_no_x"])
def test_noalloc_aliases_and_nan_rules(case):
    """x, y and z may alias; beta == 0 never reads y; alpha == 0 never reads x."""
    from warp_preconditioners_gb300 import FSAI, from_scipy, problems

    dev = torch.device("cuda:0")
    a = problems.laplacian_2d(20)
    n = a.shape[0]
    pre = FSAI(from_scipy(a, dev), max_row_size=8)
    _, fn = _entry()
    rng = np.random.default_rng(5)
    x0 = rng.normal(size=n)
    y0 = rng.normal(size=n)
    alpha, beta = 0.9, 0.4
    if case == "z_is_x":
        x = torch.as_tensor(x0, device=dev)
        y = torch.as_tensor(y0, device=dev)
        z = x
        want = _dense_apply(pre, x0, y0, alpha, beta)
    elif case == "z_is_y":
        x = torch.as_tensor(x0, device=dev)
        y = torch.as_tensor(y0, device=dev)
        z = y
        want = _dense_apply(pre, x0, y0, alpha, beta)
    elif case == "x_is_y_is_z":
        x = torch.as_tensor(x0, device=dev)
        y = z = x
        want = _dense_apply(pre, x0, x0, alpha, beta)
    elif case == "nan_y_beta0":
        beta = 0.0
        x = torch.as_tensor(x0, device=dev)
        y = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        z = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        want = _dense_apply(pre, x0, None, alpha, 0.0)
    else:  # alpha0_no_x
        alpha = 0.0
        x = None
        y = torch.as_tensor(y0, device=dev)
        z = torch.empty(n, dtype=torch.float64, device=dev)
        want = beta * y0
    for _ in range(2):  # the second call runs on the scratch the first one left
        if case in ("z_is_x", "z_is_y", "x_is_y_is_z"):
            # restore the aliased inputs before each call
            src = x0 if case != "z_is_y" else y0
            z.copy_(torch.as_tensor(src, device=dev))
            if case == "z_is_x":
                y.copy_(torch.as_tensor(y0, device=dev))
            if case == "z_is_y":
                x.copy_(torch.as_tensor(x0, device=dev))
        assert _call(fn, pre, x, y, z, alpha, beta) == 0
        torch.cuda.synchronize()
        got = z.cpu().numpy()
        assert np.isfinite(got).all()
        np.testing.assert_allclose(got, want, rtol=1e-11, atol=1e-12)


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
    torch.cuda.synchronize()
    g = pre.G.dense()
    np.testing.assert_allclose(z.cpu().numpy(), g.T @ (g @ np.ones(a.shape[0])), rtol=RTOL)
