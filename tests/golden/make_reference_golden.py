"""Golden outputs of the reference's own code, run on the host.

The reference (alecjacobson/warp-preconditioners) needs warp-lang, which is
not installable here.  This script puts the Warp emulation in
``tests/golden/warp_emu`` on ``sys.path`` (NumPy scalars, one IEEE rounding
per operation, kernels run thread by thread; see its package docstring),
imports the reference package from its source tree unmodified, builds its
preconditioners on seeded inputs and stores inputs and outputs in
``tests/golden/ref_*.npz``:

* ``ref_fsai.npz``: FSAI factors G and G^T (``FSAI.__init__``,
  warp_preconditioners/fsai.py: build kernel, pack_factor, bsr_transposed)
  of the 64 x 64 five-point Laplacian (width 8, step 1), of the assembled
  biharmonic ``Q = alpha M + K M^-1 K`` on an 8^3 jittered tet cube (widths
  8/16/48/64, steps 1/2, width 48 without a stopping tolerance, a float32
  factor at kap 3e-3, and the factor of the same Q rounded to a float32
  matrix, built in float32), and the
  fixed-support refit of the width-8 and the width-48 factor for Q at
  2 alpha (``FSAI.update``, warp_preconditioners/fsai_reuse.py).
* ``ref_block.npz``: on A = K (x) C (K the 7-point Laplacian on 6^3 nodes,
  C = R diag(1, 1, 1e-6) R^T): BlockJacobi inverses
  (warp_preconditioners/block_ilu.py), BlockILU0 factors with 3 factor sweeps
  and one 3-sweep apply, with the defaults (12 / 4 sweeps) and relaxed (6 / 2
  sweeps, relaxation 0.8), the scalarised FSAI (width 8, kap 3e-3, float32
  factor), and the block FSAI candidate's scalar factor for 2 and 4 blocks
  (float64) and 3 blocks (its default float32 storage)
  (benchmarks/block_fsai_candidate.py).
* ``ref_quality.npz``: ``FSAI.quality`` values (4 probes seed 17, 2 probes
  seed 5) on the 6^3 tet-cube Q and the 32 x 32 Laplacian with their
  factors, and the reference's Rademacher probe vectors for four seeds.
* ``ref_ops.npz``: products of the factored squared-Laplacian operator
  (warp_preconditioners/squared_laplacian.py) on the 8^3 tet cube with its
  boundary vertices constrained: an apply with aliasing-free x, y and the
  eliminated right-hand side.

Run from the repository root (needs the reference source tree; set
WARP_PRECONDITIONERS_REF to its location):

    python tests/golden/make_reference_golden.py
"""

from __future__ import annotations

import os
import sys
import time
from pathlib import Path

import numpy as np
import scipy.sparse as ss

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
REFERENCE = Path(os.environ.get("WARP_PRECONDITIONERS_REF", "/root/reference"))

sys.dont_write_bytecode = True  # never write into the reference tree
sys.path[:0] = [str(HERE / "warp_emu"), str(REFERENCE), str(REFERENCE / "benchmarks"), str(ROOT)]

import warp as wp  # noqa: E402  (the emulation)
import warp.sparse as sp  # noqa: E402

from warp_preconditioners import FSAI, BlockILU0, BlockJacobi, SquaredLaplacianOperator  # noqa: E402,I001
from block_fsai_candidate import BlockFSAI  # noqa: E402

from warp_preconditioners_gb300 import problems  # noqa: E402  (host generators only)

ALPHA = 1.0e-4


def from_scipy(a, dtype=wp.float64):
    c = ss.coo_matrix(a)
    return sp.bsr_from_triplets(a.shape[0], a.shape[1], wp.array(c.row, dtype=int),
                                wp.array(c.col, dtype=int), wp.array(c.data, dtype=dtype))


def put_csr(out, prefix, offsets, columns, values):
    out[prefix + "_off"] = np.asarray(offsets, dtype=np.int32)
    out[prefix + "_col"] = np.asarray(columns, dtype=np.int32)
    out[prefix + "_val"] = np.asarray(values)


def put_bsr(out, prefix, m):
    nnz = m.nnz
    put_csr(out, prefix, m.offsets.numpy(), m.columns.numpy()[:nnz], m.values.numpy()[:nnz])


def fsai_cases():
    out = {}
    a = problems.laplacian_2d(64)
    put_csr(out, "lap64_A", a.indptr, a.indices, a.data)
    t = time.time()
    pre = FSAI(from_scipy(a), max_row_size=8, kap_tolerance=1e-3, max_step_size=1)
    put_bsr(out, "lap64_w8s1_G", pre.G)
    put_bsr(out, "lap64_w8s1_GT", pre.GT)
    print(f"lap64 w8 s1: nnz {pre.G.nnz} ({time.time() - t:.1f} s)", flush=True)

    verts, tets, K, mass = problems.tet_cube(8)
    Q = problems.biharmonic(K, mass, ALPHA)
    put_csr(out, "cube8_Q", Q.indptr, Q.indices, Q.data)
    for width, step, kap, fdt in [(8, 1, 1e-3, None), (16, 2, 1e-3, None), (48, 1, 1e-3, None),
                                  (48, 2, 1e-3, None), (64, 1, 1e-3, None),
                                  (8, 1, 3e-3, wp.float32)]:
        t = time.time()
        pre = FSAI(from_scipy(Q), max_row_size=width, kap_tolerance=kap, max_step_size=step,
                   factor_dtype=fdt)
        tag = f"cube8_w{width}s{step}" + ("_f32" if fdt is not None else "")
        put_bsr(out, tag + "_G", pre.G)
        put_bsr(out, tag + "_GT", pre.GT)
        out[tag + "_truncated"] = np.int32(pre.truncated_rows)
        print(f"{tag}: nnz {pre.G.nnz} ({time.time() - t:.1f} s)", flush=True)

    # No stopping tolerance: every row grows until its frontier or the
    # width runs out.
    t = time.time()
    pre = FSAI(from_scipy(Q), max_row_size=48, kap_tolerance=0.0, max_step_size=1)
    put_bsr(out, "cube8_w48s1_kap0_G", pre.G)
    put_bsr(out, "cube8_w48s1_kap0_GT", pre.GT)
    out["cube8_w48s1_kap0_truncated"] = np.int32(pre.truncated_rows)
    print(f"cube8 w48 s1 kap 0: nnz {pre.G.nnz} ({time.time() - t:.1f} s)", flush=True)

    # A float32 matrix: the whole build in float32 arithmetic.
    qf = Q.astype(np.float32)
    put_csr(out, "cube8_Qf32", qf.indptr, qf.indices, qf.data)
    t = time.time()
    pre = FSAI(from_scipy(qf, wp.float32), max_row_size=16, kap_tolerance=1e-3,
               max_step_size=2)
    put_bsr(out, "cube8_f32mat_w16s2_G", pre.G)
    put_bsr(out, "cube8_f32mat_w16s2_GT", pre.GT)
    out["cube8_f32mat_w16s2_truncated"] = np.int32(pre.truncated_rows)
    print(f"cube8 float32 matrix w16 s2: nnz {pre.G.nnz} ({time.time() - t:.1f} s)", flush=True)

    # Fixed-support refit for new values on the same pattern.
    Q2 = problems.biharmonic(K, mass, 2 * ALPHA)
    put_csr(out, "cube8_Q2", Q2.indptr, Q2.indices, Q2.data)
    pre = FSAI(from_scipy(Q), max_row_size=8, kap_tolerance=1e-3, reuse_pattern=True)
    pre.update(from_scipy(Q2))
    put_bsr(out, "cube8_refit_G", pre.G)
    put_bsr(out, "cube8_refit_GT", pre.GT)
    # The same refit on the wide (width 48, step 2) supports.
    t = time.time()
    pre = FSAI(from_scipy(Q), max_row_size=48, kap_tolerance=1e-3, max_step_size=2,
               reuse_pattern=True)
    pre.update(from_scipy(Q2))
    put_bsr(out, "cube8_refit48_G", pre.G)
    put_bsr(out, "cube8_refit48_GT", pre.GT)
    print(f"cube8 refit w48 s2: nnz {pre.G.nnz} ({time.time() - t:.1f} s)", flush=True)
    np.savez_compressed(HERE / "ref_fsai.npz", **out)


def block_cases():
    out = {}
    bsr, c = problems.kron_coupling(6, kappa=1e-6, seed=0)
    nrow = bsr.shape[0] // 3
    vals = bsr.data.reshape(-1, 3, 3)
    put_csr(out, "kron6_A", bsr.indptr, bsr.indices, vals)
    rows = np.repeat(np.arange(nrow), np.diff(bsr.indptr))
    A = sp.bsr_from_triplets(nrow, nrow, wp.array(rows, dtype=int),
                             wp.array(bsr.indices, dtype=int),
                             wp.array(vals, dtype=wp.mat33d), prune_numerical_zeros=False)
    jac = BlockJacobi(A)
    out["kron6_jacobi_inverse"] = jac.inverse_diagonal.numpy().copy()
    ilu = BlockILU0(A, factor_sweeps=3, solve_sweeps=3)
    out["kron6_ilu_factors"] = ilu.factors.numpy().copy()
    out["kron6_ilu_inverse"] = ilu.inverse_diagonal.numpy().copy()
    rng = np.random.default_rng(61)
    x = rng.uniform(-1, 1, size=3 * nrow)
    y = rng.uniform(-1, 1, size=3 * nrow)
    out["kron6_x"], out["kron6_y"] = x, y
    xv = wp.array(x.reshape(-1, 3), dtype=wp.vec3d)
    yv = wp.array(y.reshape(-1, 3), dtype=wp.vec3d)
    z = wp.zeros_like(xv)
    ilu.matvec(xv, yv, z, 0.7, -0.2)
    out["kron6_ilu_apply"] = z.numpy().reshape(-1).copy()
    z = wp.zeros_like(xv)
    jac.matvec(xv, yv, z, 0.7, -0.2)
    out["kron6_jacobi_apply"] = z.numpy().reshape(-1).copy()
    # The reference's defaults (12 factor sweeps, 4 solve sweeps), and a
    # relaxed factorisation.
    for tag, kw in (("ilu_default", {}), ("ilu_relaxed", dict(factor_sweeps=6, solve_sweeps=2,
                                                                   relaxation=0.8))):
        m = BlockILU0(A, **kw)
        out[f"kron6_{tag}_factors"] = m.factors.numpy().copy()
        out[f"kron6_{tag}_inverse"] = m.inverse_diagonal.numpy().copy()
        z = wp.zeros_like(xv)
        m.matvec(xv, yv, z, 0.7, -0.2)
        out[f"kron6_{tag}_apply"] = z.numpy().reshape(-1).copy()
    pre = FSAI(A, max_row_size=8, kap_tolerance=3e-3, factor_dtype=wp.float32)
    put_bsr(out, "kron6_fsai_G", pre.G)
    put_bsr(out, "kron6_fsai_GT", pre.GT)
    for blocks in (2, 4):
        bf = BlockFSAI(A, max_blocks=blocks, factor_dtype=wp.float64)
        put_bsr(out, f"kron6_bfsai{blocks}_G", bf.G)
        put_bsr(out, f"kron6_bfsai{blocks}_GT", bf.GT)
    # Three blocks with the candidate's default float32 factor storage.
    bf = BlockFSAI(A, max_blocks=3)
    put_bsr(out, "kron6_bfsai3_f32_G", bf.G)
    put_bsr(out, "kron6_bfsai3_f32_GT", bf.GT)
    np.savez_compressed(HERE / "ref_block.npz", **out)
    print("block cases done", flush=True)


def operator_cases():
    out = {}
    verts, tets, K, mass = problems.tet_cube(8)
    side = 8
    idx = np.arange(side ** 3).reshape(side, side, side)
    inner = np.zeros((side, side, side), dtype=bool)
    inner[1:-1, 1:-1, 1:-1] = True
    free = idx[inner].astype(np.int32)
    put_csr(out, "cube8_K", K.indptr, K.indices, K.data)
    out["cube8_mass"] = mass
    out["cube8_free"] = free
    op = SquaredLaplacianOperator(from_scipy(K), wp.array(mass, dtype=wp.float64),
                                  wp.array(free, dtype=int), mass_weight=ALPHA)
    rng = np.random.default_rng(83)
    x = rng.uniform(-1, 1, size=len(free))
    y = rng.uniform(-1, 1, size=len(free))
    out["cube8_x"], out["cube8_y"] = x, y
    z = wp.zeros(len(free), dtype=wp.float64)
    op.matvec(wp.array(x, dtype=wp.float64), wp.array(y, dtype=wp.float64), z, 0.7, -0.2)
    out["cube8_sqlap_apply"] = z.numpy().copy()
    bc = rng.uniform(-1, 1, size=side ** 3)
    out["cube8_boundary"] = bc
    out["cube8_sqlap_rhs"] = op.rhs(wp.array(bc, dtype=wp.float64)).numpy().copy()
    # FSAI apply of the Q factor on the same seeded vectors.
    Q = problems.biharmonic(K, mass, ALPHA)
    pre = FSAI(from_scipy(Q), max_row_size=8)
    xq = rng.uniform(-1, 1, size=Q.shape[0])
    yq = rng.uniform(-1, 1, size=Q.shape[0])
    out["cube8_xq"], out["cube8_yq"] = xq, yq
    zq = wp.zeros(Q.shape[0], dtype=wp.float64)
    pre.matvec(wp.array(xq, dtype=wp.float64), wp.array(yq, dtype=wp.float64), zq, 0.7, -0.2)
    out["cube8_fsai_apply"] = zq.numpy().copy()
    np.savez_compressed(HERE / "ref_ops.npz", **out)
    print("operator cases done", flush=True)


def quality_cases():
    """FSAI.quality (warp_preconditioners/fsai_reuse.py:248-279) on the 6^3
    tet-cube Q (w8 factor) and the 32 x 32 Laplacian (w4 factor), with the
    reference's own probe vectors (its `probe` kernel, fsai_reuse.py:143-147)."""
    from warp_preconditioners.fsai_reuse import kernels

    out = {}
    verts, tets, K, mass = problems.tet_cube(6)
    Q = problems.biharmonic(K, mass, ALPHA)
    lap = problems.laplacian_2d(32)
    for tag, a, width in (("cube6", Q, 8), ("lap32", lap, 4)):
        put_csr(out, tag + "_A", a.indptr, a.indices, a.data)
        pre = FSAI(from_scipy(a), max_row_size=width)
        put_bsr(out, tag + "_G", pre.G)
        put_bsr(out, tag + "_GT", pre.GT)
        for probes, seed in ((4, 17), (2, 5)):
            out[f"{tag}_quality_p{probes}_s{seed}"] = np.float64(pre.quality(probes=probes,
                                                                             seed=seed))
    probe = kernels(wp.float64, wp.float64, 8)[3]
    for seed in (17, 18, 5, 123456):
        x = wp.empty(300, dtype=wp.float64)
        wp.launch(probe, 300, [seed, x])
        out[f"probe_s{seed}"] = x.numpy().copy()
    np.savez_compressed(HERE / "ref_quality.npz", **out)
    print("quality cases done", flush=True)


if __name__ == "__main__":
    which = sys.argv[1:] or ["fsai", "block", "ops", "quality"]
    if "quality" in which:
        quality_cases()
    if "block" in which:
        block_cases()
    if "ops" in which:
        operator_cases()
    if "fsai" in which:
        fsai_cases()
