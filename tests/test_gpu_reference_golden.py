"""The GPU path against outputs of the reference's own code.

``tests/golden/ref_*.npz`` hold what the reference package computes on the
same inputs (its source run unmodified on the Warp emulation,
tests/golden/make_reference_golden.py).  Integer arrays (FSAI supports,
transposes) must be equal, and so must the values: the setup kernels follow
the reference's operation order without contraction, so FSAI, refit, block
Jacobi, block ILU(0) and block FSAI factors are compared bit for bit.
Products (FSAI apply, factored operator) are compared at 1e-12 relative,
since the device sums rows in its own order with fused multiply-adds; the
block applies at 1e-9 of the largest entry (their inverse blocks carry a
1e6 condition number).
"""

import numpy as np
import pytest
import torch

from conftest import GOLDEN
from gpu_helpers import cuda, host_csr, vec

pytestmark = pytest.mark.gpu

REF_FSAI = [(8, 1, 1e-3, None), (16, 2, 1e-3, None), (48, 1, 1e-3, None), (48, 2, 1e-3, None),
            (64, 1, 1e-3, None), (8, 1, 3e-3, torch.float32)]


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.int64 if a.dtype == np.float64 else np.int32)


def _matrix(f, p, block=1):
    from warp_preconditioners_gb300.sparse import BsrMatrix

    off = torch.as_tensor(f[p + "_off"], device=cuda())
    col = torch.as_tensor(f[p + "_col"], device=cuda())
    val = torch.as_tensor(np.ascontiguousarray(f[p + "_val"]), device=cuda())
    n = len(f[p + "_off"]) - 1
    return BsrMatrix(n, n, (block, block), off, col, val)


def assert_factor_equal(m, f, p):
    off, col, val = host_csr(m)
    np.testing.assert_array_equal(off, f[p + "_off"])
    np.testing.assert_array_equal(col, f[p + "_col"])
    assert val.dtype == f[p + "_val"].dtype
    np.testing.assert_array_equal(_bits(val), _bits(f[p + "_val"]))


def _close(got, want, rtol=1e-12):
    scale = np.max(np.abs(want))
    np.testing.assert_allclose(got, want, rtol=rtol, atol=rtol * scale)


@pytest.fixture(scope="module")
def ref_fsai():
    return np.load(GOLDEN / "ref_fsai.npz")


@pytest.fixture(scope="module")
def ref_block():
    return np.load(GOLDEN / "ref_block.npz")


@pytest.fixture(scope="module")
def ref_ops():
    return np.load(GOLDEN / "ref_ops.npz")


def test_fsai_laplacian64(ref_fsai):
    from warp_preconditioners_gb300 import FSAI

    pre = FSAI(_matrix(ref_fsai, "lap64_A"), max_row_size=8, kap_tolerance=1e-3)
    assert_factor_equal(pre.G, ref_fsai, "lap64_w8s1_G")
    assert_factor_equal(pre.GT, ref_fsai, "lap64_w8s1_GT")


@pytest.mark.parametrize("width,step,kap,fdt", REF_FSAI)
def test_fsai_tet_cube_biharmonic(ref_fsai, width, step, kap, fdt):
    from warp_preconditioners_gb300 import FSAI

    pre = FSAI(_matrix(ref_fsai, "cube8_Q"), max_row_size=width, kap_tolerance=kap,
               max_step_size=step, factor_dtype=fdt)
    tag = f"cube8_w{width}s{step}" + ("_f32" if fdt is not None else "")
    assert_factor_equal(pre.G, ref_fsai, tag + "_G")
    assert_factor_equal(pre.GT, ref_fsai, tag + "_GT")
    assert pre.truncated_rows == int(ref_fsai[tag + "_truncated"])


def test_fsai_float32_matrix(ref_fsai):
    # The build in float32 arithmetic (the float instantiation of the build).
    from warp_preconditioners_gb300 import FSAI

    q = _matrix(ref_fsai, "cube8_Qf32")
    assert q.values.dtype == torch.float32
    pre = FSAI(q, max_row_size=16, kap_tolerance=1e-3, max_step_size=2)
    assert_factor_equal(pre.G, ref_fsai, "cube8_f32mat_w16s2_G")
    assert_factor_equal(pre.GT, ref_fsai, "cube8_f32mat_w16s2_GT")
    assert pre.truncated_rows == int(ref_fsai["cube8_f32mat_w16s2_truncated"])


def test_fsai_without_stopping_tolerance(ref_fsai):
    # Every row grows until its frontier or the width runs out.
    from warp_preconditioners_gb300 import FSAI

    pre = FSAI(_matrix(ref_fsai, "cube8_Q"), max_row_size=48, kap_tolerance=0.0,
               max_step_size=1)
    assert_factor_equal(pre.G, ref_fsai, "cube8_w48s1_kap0_G")
    assert_factor_equal(pre.GT, ref_fsai, "cube8_w48s1_kap0_GT")
    assert pre.truncated_rows == int(ref_fsai["cube8_w48s1_kap0_truncated"])


@pytest.mark.parametrize("width,step,tag", [(8, 1, "cube8_refit"), (48, 2, "cube8_refit48")])
def test_fsai_refit(ref_fsai, width, step, tag):
    # Width 48 runs the wide refit (a thread per row, factors in device memory).
    from warp_preconditioners_gb300 import FSAI

    pre = FSAI(_matrix(ref_fsai, "cube8_Q"), max_row_size=width, kap_tolerance=1e-3,
               max_step_size=step, reuse_pattern=True)
    pre.update(_matrix(ref_fsai, "cube8_Q2"))
    assert_factor_equal(pre.G, ref_fsai, tag + "_G")
    assert_factor_equal(pre.GT, ref_fsai, tag + "_GT")


def test_block_jacobi_and_ilu0(ref_block):
    from warp_preconditioners_gb300 import BlockILU0, BlockJacobi

    A = _matrix(ref_block, "kron6_A", block=3)
    jac = BlockJacobi(A)
    np.testing.assert_array_equal(_bits(jac.inverse_diagonal.cpu().numpy()),
                                  _bits(ref_block["kron6_jacobi_inverse"]))
    ilu = BlockILU0(A, factor_sweeps=3, solve_sweeps=3)
    np.testing.assert_array_equal(_bits(ilu.factors.cpu().numpy()),
                                  _bits(ref_block["kron6_ilu_factors"]))
    np.testing.assert_array_equal(_bits(ilu.inverse_diagonal.cpu().numpy()),
                                  _bits(ref_block["kron6_ilu_inverse"]))
    # The applies multiply by inverse blocks of C = R diag(1, 1, 1e-6) R^T,
    # whose 1e6 condition number turns the device's fused multiply-adds
    # (one rounding fewer per product than the reference) into relative
    # differences up to ~1e-10: 1e-9 of the largest entry is the bar here.
    x, y = vec(ref_block["kron6_x"]), vec(ref_block["kron6_y"])
    for op, key in ((ilu, "kron6_ilu_apply"), (jac, "kron6_jacobi_apply")):
        z = torch.empty_like(x)
        op.matvec(x, y, z, 0.7, -0.2)
        _close(z.cpu().numpy(), ref_block[key], rtol=1e-9)


@pytest.mark.parametrize("tag,fs,ss,relax", [("ilu_default", 12, 4, 1.0),
                                              ("ilu_relaxed", 6, 2, 0.8)])
def test_block_ilu0_sweeps_and_relaxation(ref_block, tag, fs, ss, relax):
    from warp_preconditioners_gb300 import BlockILU0

    A = _matrix(ref_block, "kron6_A", block=3)
    ilu = BlockILU0(A, factor_sweeps=fs, solve_sweeps=ss, relaxation=relax)
    np.testing.assert_array_equal(_bits(ilu.factors.cpu().numpy()),
                                  _bits(ref_block[f"kron6_{tag}_factors"]))
    np.testing.assert_array_equal(_bits(ilu.inverse_diagonal.cpu().numpy()),
                                  _bits(ref_block[f"kron6_{tag}_inverse"]))
    # The apply to 1e-9 of the largest entry, as above.
    x, y = vec(ref_block["kron6_x"]), vec(ref_block["kron6_y"])
    z = torch.empty_like(x)
    ilu.matvec(x, y, z, 0.7, -0.2)
    _close(z.cpu().numpy(), ref_block[f"kron6_{tag}_apply"], rtol=1e-9)


def test_scalarised_and_block_fsai(ref_block):
    from warp_preconditioners_gb300 import FSAI, BlockFSAI

    A = _matrix(ref_block, "kron6_A", block=3)
    pre = FSAI(A, max_row_size=8, kap_tolerance=3e-3, factor_dtype=torch.float32)
    assert_factor_equal(pre.G, ref_block, "kron6_fsai_G")
    assert_factor_equal(pre.GT, ref_block, "kron6_fsai_GT")
    for blocks in (2, 4):
        bf = BlockFSAI(A, max_blocks=blocks, factor_dtype=torch.float64)
        assert_factor_equal(bf.G, ref_block, f"kron6_bfsai{blocks}_G")
        assert_factor_equal(bf.GT, ref_block, f"kron6_bfsai{blocks}_GT")
    bf = BlockFSAI(A, max_blocks=3)  # the default float32 storage
    assert_factor_equal(bf.G, ref_block, "kron6_bfsai3_f32_G")
    assert_factor_equal(bf.GT, ref_block, "kron6_bfsai3_f32_GT")


def test_factored_operator_and_fsai_apply(ref_ops, ref_fsai):
    from warp_preconditioners_gb300 import FSAI, SquaredLaplacianOperator

    K = _matrix(ref_ops, "cube8_K")
    mass = vec(ref_ops["cube8_mass"])
    free = torch.as_tensor(ref_ops["cube8_free"], device=cuda())
    op = SquaredLaplacianOperator(K, mass, free, mass_weight=1e-4)
    z = torch.empty(len(free), dtype=torch.float64, device=cuda())
    op.matvec(vec(ref_ops["cube8_x"]), vec(ref_ops["cube8_y"]), z, 0.7, -0.2)
    _close(z.cpu().numpy(), ref_ops["cube8_sqlap_apply"])
    rhs = op.rhs(vec(ref_ops["cube8_boundary"]))
    _close(rhs.cpu().numpy(), ref_ops["cube8_sqlap_rhs"])
    pre = FSAI(_matrix(ref_fsai, "cube8_Q"), max_row_size=8)
    zq = torch.empty(len(ref_ops["cube8_xq"]), dtype=torch.float64, device=cuda())
    pre.matvec(vec(ref_ops["cube8_xq"]), vec(ref_ops["cube8_yq"]), zq, 0.7, -0.2)
    _close(zq.cpu().numpy(), ref_ops["cube8_fsai_apply"])


def test_quality_probes_and_value():
    # FSAI.quality against the reference's value (fsai_reuse.py:248-279) and
    # the device Rademacher probes against its probe kernel, bit for bit.
    from warp_preconditioners_gb300 import FSAI, _lib

    f = np.load(GOLDEN / "ref_quality.npz")
    x = torch.empty(300, dtype=torch.float64, device=cuda())
    for seed in (17, 18, 5, 123456):
        _lib.call("gbpc_rademacher", 300, seed, _lib.GBPC_F64, _lib.ptr(x), _lib.stream(cuda()))
        np.testing.assert_array_equal(x.cpu().numpy(), f[f"probe_s{seed}"])
    for tag, width in (("cube6", 8), ("lap32", 4)):
        pre = FSAI(_matrix(f, tag + "_A"), max_row_size=width)
        assert_factor_equal(pre.G, f, tag + "_G")
        for probes, seed in ((4, 17), (2, 5)):
            want = float(f[f"{tag}_quality_p{probes}_s{seed}"])
            got = pre.quality(probes=probes, seed=seed)
            assert abs(got - want) <= 1e-12 * want, (tag, probes, seed, got, want)
