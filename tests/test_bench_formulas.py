"""The roofline numerators bench.py reports, pinned at the C2 sizes (70^3
tet cube: n = 343,000, nnz(K) = 5,026,594 stored K entries in the C2 run,
nnz(G) = nnz(G^T) = 2,743,173), so a change to a formula shows up here
before it shows up in a benchmark line."""

import bench

N, NNZ_K, NNZ_G = 343_000, 5_026_594, 2_743_173


def test_pcg_iteration_bytes():
    # SpMV(A) for the factored operator (two K streams, both index arrays,
    # the vector reads and writes) + FSAI apply (G and G^T) + 9 n vector
    # words of the fused updates.
    spmv_k = 2 * (NNZ_K * 12 + 4 * (N + 1)) + 6 * N * 8
    fsai = 2 * NNZ_G * 12 + 2 * 4 * (N + 1) + 4 * N * 8
    assert bench.iteration_bytes(N, NNZ_K, NNZ_G, NNZ_G) == spmv_k + fsai + 9 * N * 8
    assert bench.iteration_bytes(N, NNZ_K, NNZ_G, NNZ_G) == 244_098_424


def test_pcg_fp64_flops_and_fraction():
    r = bench.pcg_fp64_roofline(N, NNZ_K, NNZ_G, NNZ_G, total_iters=1000, solve_s=1.0)
    assert r["algorithmic_flops_per_iteration"] == 2 * (2 * NNZ_K + 2 * NNZ_G) + 15 * N
    assert r["algorithmic_flops_per_iteration"] == 36_224_068
    assert abs(r["achieved"] - 36_224_068 * 1000 / 1e12) < 1e-15
    assert r["bound"] == "fp64" and r["frac"] == r["achieved"] / r["peak"]


def test_fsai_setup_roofline_record():
    r = bench.fsai_setup_roofline(4_036_474_793, 14.0)
    assert abs(r["achieved"] - 4_036_474_793 / 0.014 / 1e12) < 1e-12
    assert r["unit"] == "TFLOP/s" and r["frac"] == r["achieved"] / bench.FP64_NOMINAL_TFLOPS
