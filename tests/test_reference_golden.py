"""The oracle against outputs of the reference's own code (no GPU).

``tests/golden/ref_*.npz`` hold what the reference package computes, run
unmodified on the Warp emulation (tests/golden/make_reference_golden.py):
FSAI factors, the refit, block Jacobi inverses, block ILU(0) factors and
apply, the scalarised and block FSAI factors, and the factored
squared-Laplacian / FSAI products.  The oracle must reproduce every one of
them bit for bit.  Where the reference tree is present, its own test modules
also run on the emulation, and the cheap fixtures are regenerated and
compared with the committed ones.
"""

import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN

REF_FSAI = [(8, 1, 1e-3, None), (16, 2, 1e-3, None), (48, 1, 1e-3, None), (48, 2, 1e-3, None),
            (64, 1, 1e-3, None), (8, 1, 3e-3, np.float32)]


def _csr(o, f, p):
    return o.CSR(f[p + "_off"], f[p + "_col"], f[p + "_val"])


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.int64 if a.dtype == np.float64 else np.int32)


def assert_csr_equal(got, f, p):
    np.testing.assert_array_equal(got.offsets, f[p + "_off"])
    np.testing.assert_array_equal(got.columns, f[p + "_col"])
    assert got.values.dtype == f[p + "_val"].dtype
    np.testing.assert_array_equal(_bits(got.values), _bits(f[p + "_val"]))


@pytest.fixture(scope="module")
def ref_fsai():
    return np.load(GOLDEN / "ref_fsai.npz")


@pytest.fixture(scope="module")
def ref_block():
    return np.load(GOLDEN / "ref_block.npz")


@pytest.fixture(scope="module")
def ref_ops():
    return np.load(GOLDEN / "ref_ops.npz")


@pytest.fixture(scope="module")
def ref_quality():
    return np.load(GOLDEN / "ref_quality.npz")


def test_quality_probes_and_value(oracle, ref_quality):
    # The reference's own probe kernel output, bit for bit, and its quality
    # value to rounding (the dots are summed in a different order).
    for seed in (17, 18, 5, 123456):
        np.testing.assert_array_equal(oracle.rademacher(300, seed), ref_quality[f"probe_s{seed}"])
    for tag in ("cube6", "lap32"):
        a = _csr(oracle, ref_quality, tag + "_A")
        g, gt = _csr(oracle, ref_quality, tag + "_G"), _csr(oracle, ref_quality, tag + "_GT")
        for probes, seed in ((4, 17), (2, 5)):
            want = float(ref_quality[f"{tag}_quality_p{probes}_s{seed}"])
            got = oracle.fsai_quality(a, g, gt, probes, seed)
            assert abs(got - want) <= 1e-12 * want, (tag, got, want)


def test_fsai_laplacian64(oracle, ref_fsai):
    g, gt, _ = oracle.fsai(_csr(oracle, ref_fsai, "lap64_A"), width=8, step=1, tol=1e-3)
    assert_csr_equal(g, ref_fsai, "lap64_w8s1_G")
    assert_csr_equal(gt, ref_fsai, "lap64_w8s1_GT")


@pytest.mark.parametrize("width,step,kap,fdt", REF_FSAI)
def test_fsai_tet_cube_biharmonic(oracle, ref_fsai, width, step, kap, fdt):
    q = _csr(oracle, ref_fsai, "cube8_Q")
    g, gt, trunc = oracle.fsai(q, width=width, step=step, tol=kap, factor_dtype=fdt)
    tag = f"cube8_w{width}s{step}" + ("_f32" if fdt is not None else "")
    assert_csr_equal(g, ref_fsai, tag + "_G")
    assert_csr_equal(gt, ref_fsai, tag + "_GT")
    assert trunc == int(ref_fsai[tag + "_truncated"])


def test_fsai_float32_matrix(oracle, ref_fsai):
    q = _csr(oracle, ref_fsai, "cube8_Qf32")
    assert q.values.dtype == np.float32
    g, gt, trunc = oracle.fsai(q, width=16, step=2, tol=1e-3)
    assert_csr_equal(g, ref_fsai, "cube8_f32mat_w16s2_G")
    assert_csr_equal(gt, ref_fsai, "cube8_f32mat_w16s2_GT")
    assert trunc == int(ref_fsai["cube8_f32mat_w16s2_truncated"])


def test_fsai_without_stopping_tolerance(oracle, ref_fsai):
    q = _csr(oracle, ref_fsai, "cube8_Q")
    g, gt, trunc = oracle.fsai(q, width=48, step=1, tol=0.0)
    assert_csr_equal(g, ref_fsai, "cube8_w48s1_kap0_G")
    assert_csr_equal(gt, ref_fsai, "cube8_w48s1_kap0_GT")
    assert trunc == int(ref_fsai["cube8_w48s1_kap0_truncated"])


@pytest.mark.parametrize("width,step,tag", [(8, 1, "cube8_refit"), (48, 2, "cube8_refit48")])
def test_fsai_refit(oracle, ref_fsai, width, step, tag):
    g, _, _ = oracle.fsai(_csr(oracle, ref_fsai, "cube8_Q"), width=width, step=step)
    vals, bad_diag, bad_rows = oracle.fsai_refit(_csr(oracle, ref_fsai, "cube8_Q2"), g)
    assert bad_diag == 0 and bad_rows == 0
    np.testing.assert_array_equal(g.columns, ref_fsai[tag + "_G_col"])
    np.testing.assert_array_equal(_bits(vals), _bits(ref_fsai[tag + "_G_val"]))


def test_block_jacobi_and_ilu0(oracle, ref_block):
    off, col, val = ref_block["kron6_A_off"], ref_block["kron6_A_col"], ref_block["kron6_A_val"]
    nrow = len(off) - 1
    inv, bad = oracle.block_diag_inverse(nrow, 3, off, col, val)
    assert bad == 0
    np.testing.assert_array_equal(_bits(inv), _bits(ref_block["kron6_jacobi_inverse"]))
    fac, inv2, bad = oracle.bilu0_setup(nrow, 3, off, col, val, factor_sweeps=3)
    assert bad == 0
    np.testing.assert_array_equal(_bits(fac), _bits(ref_block["kron6_ilu_factors"]))
    np.testing.assert_array_equal(_bits(inv2), _bits(ref_block["kron6_ilu_inverse"]))
    x, y = ref_block["kron6_x"], ref_block["kron6_y"]
    z = oracle.bilu0_apply(nrow, 3, off, col, fac, inv2, 3, x, y, 0.7, -0.2)
    np.testing.assert_array_equal(_bits(z), _bits(ref_block["kron6_ilu_apply"]))
    z = oracle.block_jacobi_apply(inv, x, y, 0.7, -0.2)
    np.testing.assert_array_equal(_bits(z), _bits(ref_block["kron6_jacobi_apply"]))


@pytest.mark.parametrize("tag,fs,ss,relax", [("ilu_default", 12, 4, 1.0),
                                              ("ilu_relaxed", 6, 2, 0.8)])
def test_block_ilu0_sweeps_and_relaxation(oracle, ref_block, tag, fs, ss, relax):
    off, col, val = ref_block["kron6_A_off"], ref_block["kron6_A_col"], ref_block["kron6_A_val"]
    nrow = len(off) - 1
    fac, inv, bad = oracle.bilu0_setup(nrow, 3, off, col, val, factor_sweeps=fs,
                                       relaxation=relax)
    assert bad == 0
    np.testing.assert_array_equal(_bits(fac), _bits(ref_block[f"kron6_{tag}_factors"]))
    np.testing.assert_array_equal(_bits(inv), _bits(ref_block[f"kron6_{tag}_inverse"]))
    x, y = ref_block["kron6_x"], ref_block["kron6_y"]
    z = oracle.bilu0_apply(nrow, 3, off, col, fac, inv, ss, x, y, 0.7, -0.2)
    np.testing.assert_array_equal(_bits(z), _bits(ref_block[f"kron6_{tag}_apply"]))


def test_scalarised_and_block_fsai(oracle, ref_block):
    off, col, val = ref_block["kron6_A_off"], ref_block["kron6_A_col"], ref_block["kron6_A_val"]
    nrow = len(off) - 1
    sc = oracle.scalarize(nrow, 3, off, col, val)
    g, gt, _ = oracle.fsai(sc, width=8, step=1, tol=3e-3, factor_dtype=np.float32)
    assert_csr_equal(g, ref_block, "kron6_fsai_G")
    assert_csr_equal(gt, ref_block, "kron6_fsai_GT")
    for blocks in (2, 4):
        cols, vals, _, bad = oracle.block_fsai_setup(nrow, 3, blocks, off, col, val)
        assert bad == 0
        g = oracle.fsai_pack(3 * nrow, 3 * blocks, cols, vals)
        assert_csr_equal(g, ref_block, f"kron6_bfsai{blocks}_G")
        assert_csr_equal(oracle.transpose(g), ref_block, f"kron6_bfsai{blocks}_GT")
    # Three blocks, the candidate's default float32 storage.
    cols, vals, _, bad = oracle.block_fsai_setup(nrow, 3, 3, off, col, val)
    assert bad == 0
    g = oracle.fsai_pack(3 * nrow, 9, cols, vals)
    g = oracle.CSR(g.offsets, g.columns, g.values.astype(np.float32))
    assert_csr_equal(g, ref_block, "kron6_bfsai3_f32_G")
    assert_csr_equal(oracle.transpose(g), ref_block, "kron6_bfsai3_f32_GT")


def test_factored_operator_and_fsai_apply(oracle, ref_ops, ref_fsai):
    K = _csr(oracle, ref_ops, "cube8_K")
    mass, free = ref_ops["cube8_mass"], ref_ops["cube8_free"]
    z = oracle.sqlap_apply(K, mass, free, 1e-4, ref_ops["cube8_x"], ref_ops["cube8_y"], 0.7, -0.2)
    np.testing.assert_array_equal(_bits(z), _bits(ref_ops["cube8_sqlap_apply"]))
    # rhs(): the boundary product with the mass term off, alpha = -1, beta = 0
    z = oracle.sqlap_apply(K, mass, free, 0.0, ref_ops["cube8_boundary"], np.zeros(len(free)),
                           -1.0, 0.0, boundary=True)
    np.testing.assert_array_equal(_bits(z), _bits(ref_ops["cube8_sqlap_rhs"]))
    g, gt, _ = oracle.fsai(_csr(oracle, ref_fsai, "cube8_Q"), width=8)
    z = oracle.fsai_apply(g, gt, ref_ops["cube8_xq"], ref_ops["cube8_yq"], 0.7, -0.2)
    np.testing.assert_array_equal(_bits(z), _bits(ref_ops["cube8_fsai_apply"]))


def _runner():
    sys.path.insert(0, str(GOLDEN))
    try:
        import run_reference_tests
    finally:
        sys.path.remove(str(GOLDEN))
    return run_reference_tests


def test_reference_tests_pass_on_the_emulation():
    runner = _runner()
    if not runner.available():
        pytest.skip("reference source tree not present")
    for module in runner.MODULES:
        res = runner.run(module)
        assert res["rc"] == 0, res["output"]
        assert res["counts"].get("passed", 0) > 0, res["tail"]


def test_cheap_fixtures_regenerate(tmp_path):
    """The block and operator fixtures are what the generator writes now."""
    runner = _runner()
    if not runner.available():
        pytest.skip("reference source tree not present")
    # Run the generator's functions with its output directory redirected.
    script = (
        "import sys, runpy\n"
        "from pathlib import Path\n"
        f"g = runpy.run_path({str(GOLDEN / 'make_reference_golden.py')!r}, run_name='gen')\n"
        f"out = Path({str(tmp_path)!r})\n"
        "g['block_cases'].__globals__['HERE'] = out\n"
        "g['block_cases']()\n"
        "g['operator_cases']()\n"
    )
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, env=env,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    for name in ("ref_block.npz", "ref_ops.npz"):
        new, old = np.load(tmp_path / name), np.load(GOLDEN / name)
        assert sorted(new.files) == sorted(old.files)
        for k in old.files:
            np.testing.assert_array_equal(_bits(new[k]) if new[k].dtype.kind == "f" else new[k],
                                          _bits(old[k]) if old[k].dtype.kind == "f" else old[k])
