#!/usr/bin/env python
"""Benchmark: biharmonic smoothing on a 70^3 tet cube, setup + solve.

Workload (one step): build the factored operator (alpha M + K M^-1 K) and an
adaptive FSAI (width 8, single-entry growth, kap 1e-3) on the assembled
Q = alpha M + K M^-1 K, then solve Q u = alpha M f for four right-hand sides
(f = sin(3x) + cos(2y) z + x z, then the vertex x, y, z coordinates) with
preconditioned CG to relative residual 1e-8, all in float64 on the GPU.
Inputs are synthetic and seeded; assembly of K, M and Q happens once on the
host and is not timed (as in the reference).

Prints one JSON line.  `value` is solves/s with inputs resident on the device;
`e2e` is the same metric through the public API starting from pinned host
buffers (host->device copies of Q, K, mass and the right-hand sides and the
device->host copy of the solutions inside the timed region).

--impl reference times the reference algorithm's CPU restatement (the oracle,
all host threads) on the same workload: a bounded sample (setup plus a fixed
number of CG iterations per right-hand side) extrapolated to the iteration
count that the CPU solve needs, measured once in the warm-up.

Multi-GPU (--gpus N under torchrun): the path has no data exchange, so every
rank solves its own replica of the workload ("replicas only"); `value` sums
all ranks' solves over the slowest rank's time.
"""

from __future__ import annotations

import argparse
import collections
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "setup+solve ms and solves/s at 1e-8 rel residual; apply GB/s; p50/p99 latency"
ALPHA = 1e-4


def parse_args():
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--side", type=int, default=70, help="vertices per cube edge")
    p.add_argument("--width", type=int, default=8, help="FSAI max_row_size")
    p.add_argument("--step-size", type=int, default=1, help="FSAI max_step_size")
    p.add_argument("--method", choices=["cg", "cr"], default="cg")
    p.add_argument("--rtol", type=float, default=1e-8)
    p.add_argument("--cpu-iters", type=int, default=3000,
                   help="CG iterations per right-hand side in the CPU sample (about 2.5 s of "
                        "oracle work at 70^3 on 16 Grace cores, plus the FSAI setup)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--config", choices=["c1", "c2", "c2sweep", "c3", "c5", "gmres"], default="c2",
                   help="c2: biharmonic smoothing (default); c3: K (x) C block coupling, "
                        "every preconditioner under CG and CR; c5: serving stream")
    p.add_argument("--c3-grid", type=int, default=64)
    p.add_argument("--gmres-steps", type=int, default=300,
                   help="--config gmres: Arnoldi steps timed")
    p.add_argument("--host-loop", action="store_true",
                   help="--config gmres: host-driven loop instead of the graph (for ncu)")
    p.add_argument("--c5-requests", type=int, default=200,
                   help="requests replayed from the seed-0 stream (its first N of 2,000)")
    p.add_argument("--c5-rate", type=float, default=4.0, help="Poisson arrivals per second")
    p.add_argument("--c5-slots", type=int, default=16)
    p.add_argument("--c5-merge", type=int, default=0,
                   help="also serve with queued requests of one system merged into batched "
                        "solves of up to this many right-hand sides (0: skip that arm)")
    p.add_argument("--c5-cluster-small", action="store_true",
                   help="also serve with small systems' multi-RHS requests as one cluster "
                        "solve per right-hand side instead of the batched solver")
    p.add_argument("--c5-wide-from", type=int, default=0,
                   help="also serve with FSAI width 48 for systems of at least this many "
                        "unknowns (0: skip that arm)")
    p.add_argument("--c5-wide-step", type=int, default=2,
                   help="max_step_size of the width-48 factors of that arm")
    p.add_argument("--c5-budget-gb", type=float, default=120.0)
    p.add_argument("--c5-nmin", type=float, default=5e3)
    p.add_argument("--c5-nmax", type=float, default=5e5)
    p.add_argument("--c5-no-sequential", action="store_true",
                   help="skip the one-at-a-time float64 arm")
    p.add_argument("--no-configs", action="store_true",
                   help="skip the C1 and C3 sub-measurements of the default line")
    p.add_argument("--no-mixed", action="store_true",
                   help="skip the mixed-precision 32-RHS batched measurement")
    p.add_argument("--fp32-refinement", action="store_true",
                   help="also run float32 inner solves with float64 refinement on the 32 RHS "
                        "(does not reach float64 accuracy at 70^3; about a minute)")
    p.add_argument("--lifted", action="store_true",
                   help="also time the lifted first-order system under GMRES (the "
                        "reference's lifted-gmres method) on the first right-hand side")
    p.add_argument("--profile-iters", type=int, default=0,
                   help="profiling mode: one setup and one solve capped at this many "
                        "iterations, no timing (for ncu launch lists)")
    p.add_argument("--profile-fsai", type=int, default=0,
                   help="profiling mode: two FSAI setups of this width (and --step-size) "
                        "on the --side system's Q, setup times only (for ncu)")
    return p.parse_args()


def build_problem(side):
    from warp_preconditioners_gb300 import problems

    t0 = time.perf_counter()
    verts, tets, K, mass = problems.tet_cube(side)
    Q = problems.biharmonic(K, mass, ALPHA)
    rhs = problems.smoothing_rhs(verts, mass, ALPHA)
    return dict(verts=verts, K=K, mass=mass, Q=Q, rhs=rhs, n=K.shape[0], ntets=len(tets),
                assembly_s=time.perf_counter() - t0)


def iteration_bytes(n, nnz_k, nnz_g, nnz_gt):
    """Algorithmic bytes of one float64 PCG iteration (factored operator + FSAI)."""
    spmv_k = 2 * (nnz_k * 12 + 4 * (n + 1)) + 5 * n * 8 + n * 8
    fsai = (nnz_g + nnz_gt) * 12 + 2 * 4 * (n + 1) + 4 * n * 8
    vectors = 9 * n * 8
    return spmv_k + fsai + vectors


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = []
        for line in Path(self.file.name).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def cpu_baseline_sample(prob, width, step_size, method, cpu_iters, iterations_per_rhs,
                        count_flops=True):
    """Oracle (CPU restatement) on the host cores: FSAI setup + cpu_iters iterations."""
    from oracle import oracle

    o = oracle
    Q, K, mass = prob["Q"], prob["K"], prob["mass"]
    qc = o.CSR(Q.indptr, Q.indices, Q.data)
    kc = o.CSR(K.indptr, K.indices, K.data)
    t0 = time.perf_counter()
    g, gt, _ = o.fsai(qc, width=width, step=step_size, tol=1e-3)
    setup = time.perf_counter() - t0
    A = o.Operator.sqlap(kc, mass, ALPHA)
    M = o.Operator.fsai(g, gt)
    t0 = time.perf_counter()
    _, it, _, _ = o.krylov(method, A, prob["rhs"][0], M=M, tol=0.0, maxiter=cpu_iters)
    per_iter = (time.perf_counter() - t0) / max(it, 1)
    total = setup + per_iter * sum(iterations_per_rhs)
    # Operation count of the same setup (untimed: the counting run is separate).
    flops = None
    if count_flops:
        flops, _, _ = o.fsai_setup_flops(qc, width=width, step=step_size, tol=1e-3)
    return dict(setup_s=setup, per_iteration_s=per_iter, total_s=total, threads=o.num_threads(),
                iters_sampled=it, setup_flops=flops, factor=(g, gt))


def factor_parity(pre, g_or, gt_or):
    """GPU factor (the one the timed steps built) against the oracle's factor of
    the same Q: integer arrays compared exactly, values bit for bit and by the
    largest relative difference."""
    out = {}
    for name, dev_m, host in (("G", pre.G, g_or), ("GT", pre.GT, gt_or)):
        off = dev_m.offsets.cpu().numpy()
        col = dev_m.columns.cpu().numpy()
        val = dev_m.values.cpu().numpy()
        pattern = bool(np.array_equal(off, host.offsets))
        columns = pattern and bool(np.array_equal(col, host.columns))
        if columns:
            same = int(np.count_nonzero(val.view(np.int64) == host.values.view(np.int64)))
            rel = float(np.max(np.abs(val - host.values) / np.maximum(np.abs(host.values),
                                                                       np.finfo(float).tiny)))
        else:
            same, rel = 0, None
        out[name] = {"pattern_equal": pattern, "columns_equal": columns, "nnz": int(col.size),
                     "values_bit_equal": same, "max_rel_diff": rel}
    out["pattern_equal"] = out["G"]["pattern_equal"] and out["GT"]["pattern_equal"]
    out["columns_equal"] = out["G"]["columns_equal"] and out["GT"]["columns_equal"]
    out["max_rel_diff"] = max((out[k]["max_rel_diff"] or 0.0) if out[k]["columns_equal"]
                              else float("inf") for k in ("G", "GT"))
    out["bar"] = "pattern and columns exact; values within 1e-12 relative"
    out["pass"] = bool(out["columns_equal"] and out["max_rel_diff"] <= 1e-12)
    return out


def run_reference(args, prob):
    """The CPU restatement of the reference algorithm, all host threads."""
    from oracle import oracle

    threads = oracle.num_threads()
    # Warm-up: one full CPU solve of the first right-hand side to learn the
    # CPU iteration count used to extrapolate the bounded timed samples.
    Q, K, mass = prob["Q"], prob["K"], prob["mass"]
    qc = oracle.CSR(Q.indptr, Q.indices, Q.data)
    kc = oracle.CSR(K.indptr, K.indices, K.data)
    g, gt, _ = oracle.fsai(qc, width=args.width, step=args.step_size, tol=1e-3)
    A = oracle.Operator.sqlap(kc, mass, ALPHA)
    M = oracle.Operator.fsai(g, gt)
    full_iters = []
    for k in range(min(args.warmup, 1)):
        _, it, _, _ = oracle.krylov(args.method, A, prob["rhs"][k], M=M, tol=args.rtol,
                                    maxiter=200000)
        full_iters.append(it)
    if not full_iters:
        _, it, _, _ = oracle.krylov(args.method, A, prob["rhs"][0], M=M, tol=args.rtol,
                                    maxiter=200000)
        full_iters.append(it)
    its = [full_iters[0]] * 4
    samples, measured = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        s = cpu_baseline_sample(prob, args.width, args.step_size, args.method, args.cpu_iters, its,
                                count_flops=False)
        measured.append(time.perf_counter() - t0)
        samples.append(s["total_s"])
    t = statistics.median(samples)
    value = 4.0 / t
    frac = min(1.0, args.cpu_iters / float(sum(its)))
    sample = (f"FSAI w{args.width} setup + {args.cpu_iters} PCG iterations of one RHS per step "
              f"({frac:.1%} of the step's {sum(its)} iterations), extrapolated to "
              f"{full_iters[0]} iterations x 4 RHS (iteration count from one full CPU solve in "
              f"warm-up)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args, prob),
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads,
                         "kind": "port, extrapolated", "sample": sample,
                         "sampled_fraction": frac,
                         "measured_ms_per_step": statistics.median(measured) * 1e3},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(args, prob):
    Q = prob["Q"]
    return {
        "workload": f"biharmonic smoothing (alpha M + K M^-1 K) u = alpha M f on a {args.side}^3 "
                    f"jittered tet cube; FSAI w{args.width} step {args.step_size} kap 1e-3 on the "
                    f"assembled Q; factored operator; {args.method.upper()} to {args.rtol:g}; "
                    f"4 RHS; float64",
        "n": prob["n"], "tets": prob["ntets"], "nnz_K": int(prob["K"].nnz), "nnz_Q": int(Q.nnz),
        "fsai_width": args.width, "max_step_size": args.step_size, "kap_tolerance": 1e-3,
        "solver": args.method, "rhs": 4, "rel_tol": args.rtol,
        "l2": "inputs larger than L2 (Q values+columns %.0f MB > 129 MB)" % (Q.nnz * 12 / 1e6),
        "parallelism": f"replicas x{args.gpus}",
    }


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return
        prob = build_problem(args.side)
        run_reference(args, prob)
        return

    import torch

    from warp_preconditioners_gb300 import FSAI, SquaredLaplacianOperator, from_scipy, linear

    if args.config == "c3":
        if rank == 0:
            print(json.dumps(run_c3(args, torch.device("cuda", local))), flush=True)
        return
    if args.config == "c5":
        if rank == 0:
            print(json.dumps(run_c5(args, torch.device("cuda", local))), flush=True)
        return
    if args.config == "gmres":
        if rank == 0:
            print(json.dumps(run_gmres_steps(args, torch.device("cuda", local))), flush=True)
        return
    if args.config == "c1":
        if rank == 0:
            print(json.dumps(run_c1(args, torch.device("cuda", local))), flush=True)
        return
    if args.config == "c2sweep":
        if rank == 0:
            print(json.dumps(run_c2_sweep(args, torch.device("cuda", local))), flush=True)
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    prob = build_problem(args.side)
    n = prob["n"]
    Q = from_scipy(prob["Q"], dev)
    K = from_scipy(prob["K"], dev)
    mass = torch.as_tensor(prob["mass"], device=dev)
    free = torch.arange(n, dtype=torch.int32, device=dev)
    rhs = torch.as_tensor(prob["rhs"], device=dev).contiguous()
    b = torch.empty(n, dtype=torch.float64, device=dev)
    xs = torch.zeros((4, n), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def one_step(Qm, Km, massv, rhsv, out, rec=None):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        op = SquaredLaplacianOperator(Km, massv, free, mass_weight=ALPHA)
        pre = FSAI(Qm, max_row_size=args.width, max_step_size=args.step_size,
                   kap_tolerance=1e-3)
        ev[0].record(stream)
        solver = linear.Solver(args.method, op, pre)
        its = []
        for k in range(4):
            b.copy_(rhsv[k])
            out[k].zero_()
            nit, rr, _ = solver.run(b, out[k], tol=args.rtol, maxiter=100000)
            its.append(nit.clone())
        ev[1].record(stream)
        if rec is not None:
            rec.append((ev, its, pre))
        return pre

    if args.profile_fsai > 0:
        for _ in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            pre = FSAI(Q, max_row_size=args.profile_fsai, max_step_size=args.step_size,
                       kap_tolerance=1e-3)
            torch.cuda.synchronize()
            print(json.dumps({"profile_fsai": args.profile_fsai, "step": args.step_size, "n": n,
                              "setup_ms": (time.perf_counter() - t0) * 1e3,
                              "fsai_nnz": pre.G.nnz}), flush=True)
        return
    if args.profile_iters > 0:
        op = SquaredLaplacianOperator(K, mass, free, mass_weight=ALPHA)
        pre = FSAI(Q, max_row_size=args.width, max_step_size=args.step_size, kap_tolerance=1e-3)
        # Host-driven loop: kernels inside a graph with conditional nodes cannot
        # be profiled individually.
        solver = linear.Solver(args.method, op, pre, use_cuda_graph=False)
        nit, _, _ = solver.run(rhs[0], xs[0], tol=args.rtol, maxiter=args.profile_iters)
        torch.cuda.synchronize()
        print(json.dumps({"profile_iters": int(nit.item()), "n": n, "fsai_nnz": pre.G.nnz}))
        return

    for _ in range(args.warmup):
        one_step(Q, K, mass, rhs, xs)
    torch.cuda.synchronize()

    recs = []
    with ClockSampler(local) as clocks:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(args.steps):
            one_step(Q, K, mass, rhs, xs, recs)
        end.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    value, elapsed_ms = replica_aggregate(start.elapsed_time(end), 4.0 * args.steps, dist, dev)
    ms_per_step = elapsed_ms / args.steps
    solve_ms = [r[0][0].elapsed_time(r[0][1]) for r in recs]
    setup_ms = [ms_per_step - s for s in solve_ms]
    iters = [[int(i.item()) for i in r[1]] for r in recs]

    # Accuracy of the last step against the assembled Q (float64, host).
    qh = prob["Q"]
    sols = xs.cpu().numpy()
    relres = [float(np.linalg.norm(prob["rhs"][k] - qh @ sols[k]) / np.linalg.norm(prob["rhs"][k]))
              for k in range(4)]
    absq = abs(qh)
    berr = [float(np.max(np.abs(prob["rhs"][k] - qh @ sols[k])
                         / np.maximum(absq @ np.abs(sols[k]) + np.abs(prob["rhs"][k]),
                                      np.finfo(float).tiny))) for k in range(4)]
    pre = recs[-1][2]
    nnz_g, nnz_gt = pre.G.nnz, pre.GT.nnz
    total_iters = sum(sum(i) for i in iters)
    solve_total_s = sum(solve_ms) / 1e3
    it_bytes = iteration_bytes(n, prob["K"].nnz, nnz_g, nnz_gt)

    with open(ROOT / "MEASURED_PEAKS.json") as f:
        peaks = json.load(f)
    peak = float(peaks["hbm_gbs"])
    achieved = it_bytes * total_iters / solve_total_s / 1e9

    apply = measure_applies(
        pre, lambda: FSAI(Q, max_row_size=args.width, max_step_size=args.step_size,
                          kap_tolerance=1e-3), K, mass, free, n, dev,
        make_low=lambda: FSAI(Q, max_row_size=args.width, max_step_size=args.step_size,
                              kap_tolerance=1e-3, factor_dtype=torch.bfloat16,
                              apply_dtype=torch.float32))
    traffic = read_traffic()
    fp64_peak = measure_fp64_peak(dev)

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded jittered tet cube; P1 cotangent stiffness; lumped mass)",
        "config": workload_config(args, prob),
        "setup_ms": statistics.median(setup_ms), "solve_ms": statistics.median(solve_ms),
        "iterations": iters[-1], "backward_error": berr,
        "host_recomputed_relres": relres,
        "accuracy_note": "stopping test is the recursive residual (as warp.optim.linear); "
                         "b - Q x recomputed in float64 on the host is dominated by cancellation "
                         "for this operator, so the componentwise backward error max|b-Qx|/"
                         "(|Q||x|+|b|) is the accuracy measure",
        "fsai_nnz": nnz_g,
        "roofline": {
            "bound": "hbm", "unit": "GB/s", "kernel": "PCG iteration (factored operator + FSAI "
            "apply + fused updates), averaged over the timed solves",
            "achieved": achieved, "peak": peak, "frac": achieved / peak,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
            "algorithmic_bytes_per_iteration": it_bytes,
            "traffic": traffic,
        },
        "roofline_fp64": pcg_fp64_roofline(n, prob["K"].nnz, nnz_g, nnz_gt, total_iters,
                                           solve_total_s, fp64_peak),
        "fp64_peak": fp64_peak,
        "apply_gbps": apply,
        "gpu_launches": launch_count(iters, args.width),
    }
    clk = clocks.summary()
    line["clocks"] = clk
    if not args.no_e2e:
        line["e2e"] = run_e2e(args, prob, dev, one_step, world, dist)
    if not args.no_mixed:
        line["mixed_batched"] = run_mixed_batched(args, prob, Q, K, mass, free, dev)
    if not args.no_mixed:
        line["batched_rhs4"] = measure_batched_rhs4(args, prob, Q, K, mass, dev, ms_per_step)
        line["f32_apply_rhs4"] = measure_f32_apply_rhs4(args, prob, Q, K, mass, free, dev,
                                                        ms_per_step)
    if not args.no_mixed:
        line["wide_fsai"] = measure_wide_fsai(args, prob, Q, K, mass, free, dev, ms_per_step)
        line["multi_system"] = measure_multi_system(dev)
        line["multi_system_small"] = measure_multi_system(dev, sides=(17, 18, 19, 20) * 8)
    if not args.no_configs:
        # The reference's CPU-runnable case and its block-coupling benchmark,
        # measured in the same run (their own configs: --config c1 / c3).
        line["c1"] = run_c1(args, dev)
        line["c3"] = run_c3(args, dev)
    line["refit"] = measure_refit(args, prob, Q, dev)
    line["assembly"] = measure_assembly(prob, dev)
    if args.lifted:
        line["lifted_gmres"] = measure_lifted_gmres(args, prob, dev)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline_sample(prob, args.width, args.step_size, args.method, args.cpu_iters,
                                 iters[-1])
        line["cpu_baseline"] = {
            "value": 4.0 / cb["total_s"], "unit": "solves/s", "cores": cb["threads"],
            "kind": "port, extrapolated",
            "sample": (f"oracle FSAI w{args.width} setup ({cb['setup_s']:.2f} s) + "
                       f"{cb['iters_sampled']} PCG iterations ({cb['per_iteration_s'] * 1e3:.2f} "
                       f"ms each) on one RHS, extrapolated to the GPU's iteration counts "
                       f"{iters[-1]}"),
            "sampled_fraction": min(1.0, cb["iters_sampled"] / float(sum(iters[-1]))),
        }
        line["fsai_setup_roofline"] = fsai_setup_roofline(cb["setup_flops"],
                                                          line["refit"]["setup_ms"], fp64_peak)
        line["parity"] = factor_parity(pre, *cb["factor"])
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


FP64_NOMINAL_TFLOPS = 1.25  # GB300 nominal FP64, used only when the probe fails


def measure_fp64_peak(dev, iters=20000):
    """FP64 FMA throughput of this GPU, measured live: libgbpc's
    gbpc_fma_probe (8 independent FMA chains per thread, 8 CTAs of 256
    threads per SM) timed with CUDA events on the launching stream, best of
    3 after a warm-up.  TFLOP/s counts a multiply-add as 2 flops."""
    import ctypes

    import torch

    from warp_preconditioners_gb300 import _lib

    ctas = 152 * 8
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    st = _lib.stream(dev)
    stream = torch.cuda.current_stream(dev)
    _lib.call("gbpc_fma_probe", 100, ctas, _lib.ptr(out), st)
    best = None
    for _ in range(3):
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record(stream)
        _lib.call("gbpc_fma_probe", ctypes.c_int64(iters), ctas, _lib.ptr(out), st)
        e.record(stream)
        torch.cuda.synchronize(dev)
        t = s.elapsed_time(e) / 1e3
        best = t if best is None else min(best, t)
    fmas = ctas * 256 * 8 * iters
    return {"tflops": 2 * fmas / best / 1e12, "fma_per_s": fmas / best, "ms": best * 1e3,
            "how": f"gbpc_fma_probe: {ctas} CTAs x 256 threads x 8 chains x {iters} FMAs, "
                   "CUDA events, best of 3"}


def _fp64_peak(peak):
    if peak:
        return peak["tflops"], "measured in this run (gbpc_fma_probe, FP64 FMA chains)"
    return FP64_NOMINAL_TFLOPS, "GB300 nominal FP64 (fallback: the probe did not run)"


def pcg_fp64_roofline(n, nnz_k, nnz_g, nnz_gt, total_iters, solve_s, peak=None):
    """The same timed iterations against FP64 arithmetic (a multiply-add is 2
    flops): 2 per stored entry of the two K products, of G and of G^T, and
    15 n for the epilogues, the x/r/p updates and the three dot products."""
    flops = 2 * (2 * nnz_k + nnz_g + nnz_gt) + 15 * n
    achieved = flops * total_iters / solve_s / 1e12
    p, src = _fp64_peak(peak)
    return {"bound": "fp64", "unit": "TFLOP/s", "algorithmic_flops_per_iteration": flops,
            "achieved": achieved, "peak": p, "frac": achieved / p, "peak_source": src}


def fsai_setup_roofline(flops, setup_ms, peak=None):
    """FP64 roofline of the FSAI setup: the oracle's exact operation count of
    the same setup (each separately rounded multiply, add, divide, square
    root; the reference evaluates without contraction) over the GPU
    constructor's CUDA-event time (build, pack, transpose, operator copies)."""
    achieved = flops / (setup_ms * 1e-3) / 1e12
    p, src = _fp64_peak(peak)
    return {"bound": "fp64", "unit": "TFLOP/s", "flops": flops, "setup_ms": setup_ms,
            "achieved": achieved, "peak": p, "frac": achieved / p, "peak_source": src}


def replica_aggregate(elapsed_ms, local_solves, dist, device):
    """Whole-job throughput of independent replicas: every rank's solves over
    the slowest rank's time (max over ranks)."""
    import torch

    if dist is None:
        return local_solves / (elapsed_ms / 1e3), elapsed_ms
    t = torch.tensor([elapsed_ms, float(local_solves)], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    tot = t.clone()
    dist.all_reduce(tot, op=dist.ReduceOp.SUM)
    return float(tot[1]) / (float(mx[0]) / 1e3), float(mx[0])


def run_mixed_batched(args, prob, Q, K, mass, free, dev, k=32):
    """32 seeded U[-1,1] right-hand sides of the same system: mixed-precision
    batched solve (float32 inner PCG on the factored operator with a bfloat16
    FSAI factor, float64 refinement) against 32 sequential plain float64
    solves, each including its setup."""
    import torch

    from warp_preconditioners_gb300 import FSAI, SquaredLaplacianOperator, batched, linear

    n = prob["n"]
    b_np = np.stack([np.random.default_rng(s).uniform(-1, 1, n) for s in range(k)], 1)
    B = torch.as_tensor(b_np, device=dev).contiguous()

    def plain():
        op = SquaredLaplacianOperator(K, mass, free, mass_weight=ALPHA)
        pre = FSAI(Q, max_row_size=args.width, max_step_size=args.step_size, kap_tolerance=1e-3)
        solver = linear.Solver("cg", op, pre)
        xs = torch.zeros((k, n), dtype=torch.float64, device=dev)
        b = torch.empty(n, dtype=torch.float64, device=dev)
        its = []
        for j in range(k):
            b.copy_(B[:, j])
            nit, _, _ = solver.run(b, xs[j], tol=args.rtol, maxiter=100000)
            its.append(nit)
        return xs, its

    def batch64(width=args.width, step=args.step_size):
        pre = FSAI(Q, max_row_size=width, max_step_size=step, kap_tolerance=1e-3)
        bs = batched.BatchedSolver(K, mass, ALPHA, pre)
        X = torch.zeros_like(B)
        nit, _ = bs.solve(B, X, tol=args.rtol, maxiter=100000)
        return X, nit.clone()

    def batch_f32m(factor_dtype, width=args.width, step=args.step_size):
        # The batched operator narrows the float32 factor to factor_dtype itself.
        pre = FSAI(Q, max_row_size=width, max_step_size=step, kap_tolerance=1e-3,
                   factor_dtype=torch.float32)
        bs = batched.BatchedSolver(K, mass, ALPHA, pre, factor_dtype=factor_dtype,
                                   apply_dtype=torch.float32)
        X = torch.zeros_like(B)
        nit, _ = bs.solve(B, X, tol=args.rtol, maxiter=100000)
        return X, nit.clone()

    def mixed():
        pre = FSAI(Q, max_row_size=args.width, max_step_size=args.step_size, kap_tolerance=1e-3)
        ms = batched.MixedPrecisionSolver(K, mass, ALPHA, pre, torch.bfloat16)
        X = torch.zeros_like(B)
        outer, inner = ms.solve(B, X, tol_outer=1e-12, tol_inner=1e-3, max_outer=8)
        return X, outer, inner

    def timed(fn):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        out = fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), out

    batch64()  # warm-up (graph capture paths)
    batch_f32m(torch.bfloat16)
    t_plain, (xs, its) = timed(plain)
    t_batch, (Xb, nitb) = timed(batch64)
    low = {dt: timed(lambda: batch_f32m(dt)) for dt in (torch.bfloat16, torch.float32)}
    # The same batched solves with the width-48, step-2 factor.
    batch64(48, 2)
    batch_f32m(torch.bfloat16, 48, 2)
    wide = {"fp64": timed(lambda: batch64(48, 2)),
            "bf16_f32apply": timed(lambda: batch_f32m(torch.bfloat16, 48, 2))}
    if args.fp32_refinement:
        t_mixed, (Xm, outer, inner) = timed(mixed)
    qh = prob["Q"]
    absq = abs(qh)
    x_p = xs.cpu().numpy().T

    def quality(x):
        berr, rel = [], []
        for j in range(k):
            den = absq @ np.abs(x[:, j]) + np.abs(b_np[:, j])
            berr.append(float(np.max(np.abs(b_np[:, j] - qh @ x[:, j]) / den)))
            rel.append(float(np.linalg.norm(x[:, j] - x_p[:, j]) / np.linalg.norm(x_p[:, j])))
        return max(berr), max(rel)

    berr_p, _ = quality(x_p)
    berr_b, rel_b = quality(Xb.cpu().numpy())
    out = {
        "workload": f"{k} seeded U[-1,1] RHS of the {args.side}^3 smoothing system; setup + solve",
        "plain_fp64_sequential_ms": t_plain, "plain_solves_per_s": k / (t_plain / 1e3),
        "plain_iterations_max": int(max(int(i.item()) for i in its)),
        "backward_error_plain_max": berr_p,
        "batched_fp64": {
            "solver": "one batched PCG for all %d RHS (float64 operator, vectors, FSAI w%d)"
                      % (k, args.width),
            "ms": t_batch, "solves_per_s": k / (t_batch / 1e3), "speedup": t_plain / t_batch,
            "iterations_max": int(nitb.max().item()), "backward_error_max": berr_b,
            "rel_diff_vs_plain_max": rel_b},
    }
    for dt, (t_low, (Xl, nitl)) in low.items():
        berr_l, rel_l = quality(Xl.cpu().numpy())
        name = "bf16" if dt == torch.bfloat16 else "f32"
        out[f"batched_f32_apply_{name}"] = {
            "solver": (f"one batched float64 PCG for all {k} RHS with the FSAI factor stored in "
                       f"{name} and applied in float32 (float64 operator, recurrences and dots)"),
            "ms": t_low, "solves_per_s": k / (t_low / 1e3), "speedup": t_plain / t_low,
            "speedup_vs_batched_fp64": t_batch / t_low,
            "iterations_max": int(nitl.max().item()), "backward_error_max": berr_l,
            "rel_diff_vs_plain_max": rel_l}
    for name, (t_w, (Xw, nitw)) in wide.items():
        berr_w, rel_w = quality(Xw.cpu().numpy())
        out[f"batched_w48_step2_{name}"] = {
            "solver": (f"one batched float64 PCG for all {k} RHS with FSAI width 48, step 2"
                       + (", the factor stored in bf16 and applied in float32"
                          if name != "fp64" else "")),
            "ms": t_w, "solves_per_s": k / (t_w / 1e3), "speedup": t_plain / t_w,
            "speedup_vs_batched_fp64": t_batch / t_w,
            "iterations_max": int(nitw.max().item()), "backward_error_max": berr_w,
            "rel_diff_vs_plain_max": rel_w}
    if args.fp32_refinement:
        berr_m, rel_m = quality(Xm.cpu().numpy())
        out["float32_refinement"] = {
            "solver": "inner float32 PCG (float32 factored operator, bfloat16 FSAI, float64 "
                      "dots), float64 refinement, 8 outer steps max",
            "ms": t_mixed, "speedup": t_plain / t_mixed, "outer_max": int(max(outer)),
            "inner_max": int(max(inner)), "backward_error_max": berr_m,
            "rel_diff_vs_plain_max": rel_m}
    return out


def _step_variant(args, prob, Q, K, mass, free, dev, ms_per_step, pre_kw, solver_kw):
    """The default step (setup + 4 sequential CG solves through linear.Solver)
    with extra FSAI / Solver keyword arguments; CUDA-event median of 3 steps,
    iteration counts and per-RHS backward error against the assembled Q."""
    import torch

    from warp_preconditioners_gb300 import FSAI, SquaredLaplacianOperator, linear

    n = prob["n"]
    rhs = torch.as_tensor(prob["rhs"], device=dev).contiguous()
    b = torch.empty(n, dtype=torch.float64, device=dev)
    xs = torch.zeros((4, n), dtype=torch.float64, device=dev)

    kw = dict(max_row_size=args.width, max_step_size=args.step_size, kap_tolerance=1e-3)
    kw.update(pre_kw)

    def step():
        op = SquaredLaplacianOperator(K, mass, free, mass_weight=ALPHA)
        pre = FSAI(Q, **kw)
        solver = linear.Solver(args.method, op, pre, **solver_kw)
        its = []
        for j in range(4):
            b.copy_(rhs[j])
            xs[j].zero_()
            nit, _, _ = solver.run(b, xs[j], tol=args.rtol, maxiter=100000)
            its.append(nit.clone())
        return its

    step()
    times = []
    for _ in range(3):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        its = step()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    t = statistics.median(times)
    qh = prob["Q"]
    sols = xs.cpu().numpy()
    absq = abs(qh)
    berr = [float(np.max(np.abs(prob["rhs"][j] - qh @ sols[j])
                         / (absq @ np.abs(sols[j]) + np.abs(prob["rhs"][j]))))
            for j in range(4)]
    setups = []
    for _ in range(3):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        FSAI(Q, **kw)
        e1.record()
        torch.cuda.synchronize()
        setups.append(e0.elapsed_time(e1))
    return {"ms_per_step": t, "solves_per_s": 4e3 / t, "speedup_vs_drop_in": ms_per_step / t,
            "setup_ms": statistics.median(setups),
            "iterations": [int(i.item()) for i in its], "backward_error_max": max(berr)}


def measure_wide_fsai(args, prob, Q, K, mass, free, dev, ms_per_step):
    """The default step with the wide factors the reference's sweep uses
    (width 48, steps 1 and 2): fewer CG iterations for a longer setup."""
    import torch

    out = {}
    for step in (1, 2):
        out[f"w48_step{step}"] = _step_variant(args, prob, Q, K, mass, free, dev, ms_per_step,
                                               dict(max_row_size=48, max_step_size=step), {})
    for name, dt in (("bf16", torch.bfloat16), ("f32", torch.float32)):
        out[f"w48_step2_{name}_f32apply"] = _step_variant(
            args, prob, Q, K, mass, free, dev, ms_per_step,
            dict(max_row_size=48, max_step_size=2, factor_dtype=dt, apply_dtype=torch.float32),
            {})
    out["solver"] = ("the default step (FSAI setup + 4 sequential CG solves) with "
                     "FSAI(Q, max_row_size=48, max_step_size=1 or 2, kap_tolerance=1e-3); "
                     "*_f32apply: the step-2 factor stored in bf16 / f32 and applied in float32 "
                     "(operator, recurrences and dots float64)")
    return out


def measure_f32_apply_rhs4(args, prob, Q, K, mass, free, dev, ms_per_step):
    """The default step with the FSAI factor applied in float32 (stored in
    bfloat16 or float32), everything else float64."""
    import torch

    out = {}
    for name, dt in (("bf16", torch.bfloat16), ("f32", torch.float32)):
        out[name] = _step_variant(args, prob, Q, K, mass, free, dev, ms_per_step,
                                  dict(apply_dtype=torch.float32, factor_dtype=dt), {})
    out["solver"] = ("the default step (setup + 4 sequential CG solves) with FSAI(..., "
                     "apply_dtype=torch.float32): factor stored in bf16 / f32 and applied in "
                     "float32; operator, recurrences and dots float64")
    return out


def measure_refit(args, prob, Q, dev):
    """Fixed-support numeric refit (FSAI.update, fsai_reuse.py) against a full
    adaptive setup: the refit takes Q with alpha doubled (same pattern, new
    values; host assembly untimed).  CUDA-event medians of 3."""
    import torch

    from warp_preconditioners_gb300 import FSAI, from_scipy, problems

    Q2 = from_scipy(problems.biharmonic(prob["K"], prob["mass"], 2 * ALPHA), dev)

    def timed(fn):
        out = []
        for _ in range(3):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            out.append(e0.elapsed_time(e1))
        return statistics.median(out)

    kw = dict(max_row_size=args.width, max_step_size=args.step_size, kap_tolerance=1e-3)
    setup_ms = timed(lambda: FSAI(Q, **kw))
    pre = FSAI(Q, reuse_pattern=True, **kw)
    mats = [Q2, Q]
    state = {"i": 0}

    def refit():
        pre.update(mats[state["i"] % 2])
        state["i"] += 1

    refit_ms = timed(refit)
    return {"matrix": f"Q with alpha {ALPHA:g} -> {2 * ALPHA:g} (same pattern)",
            "setup_ms": setup_ms, "refit_ms": refit_ms, "setup_over_refit": setup_ms / refit_ms}


def measure_multi_system(dev, sides=tuple(range(17, 38, 2)) + (18, 24, 30, 36, 22), tol=1e-8):
    """Many independent smoothing systems of uneven size in one launch, two
    ways -- multi.MultiSystemSolver (block-diagonal operator and FSAI,
    per-system scalars and stopping tests, every product over all systems)
    and multi.ClusterSolver (one thread-block cluster per system, each with
    its own operators) -- against the same systems solved one at a time
    with the drop-in float64 solver.  Tet cubes of the given sides, FSAI
    w8, first right-hand side, CG to `tol`; operators and factors built
    beforehand, solve time only, CUDA-event medians of 3."""
    import torch

    from warp_preconditioners_gb300 import FSAI, SquaredLaplacianOperator, from_scipy, linear, problems
    from warp_preconditioners_gb300.multi import MultiSystemSolver
    from warp_preconditioners_gb300.sparse import block_diag

    systems = []
    for side in sides:
        verts, _, Kh, mh = problems.tet_cube(side)
        Qh = problems.biharmonic(Kh, mh, ALPHA)
        systems.append((from_scipy(Kh, dev), from_scipy(Qh, dev),
                        torch.as_tensor(mh, device=dev),
                        torch.as_tensor(problems.smoothing_rhs(verts, mh, ALPHA)[0], device=dev)))
    sizes = [s[0].nrow for s in systems]

    def timed(fn):
        out = []
        for _ in range(3):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r = fn()
            e1.record()
            torch.cuda.synchronize()
            out.append(e0.elapsed_time(e1))
        return statistics.median(out), r

    solo = []
    for K, Q, m, b in systems:
        n = K.nrow
        op = SquaredLaplacianOperator(K, m, torch.arange(n, dtype=torch.int32, device=dev),
                                      mass_weight=ALPHA)
        solver = linear.Solver("cg", op, FSAI(Q, max_row_size=8))
        x = torch.zeros(n, dtype=torch.float64, device=dev)
        solo.append((op, solver, b, x))

    def run_solo():
        its = []
        for _, solver, b, x in solo:
            x.zero_()
            nit, _, _ = solver.run(b, x, tol=tol, maxiter=100000)
            its.append(nit)
        return its

    run_solo()
    t_solo, its_solo = timed(run_solo)
    Kb = block_diag([s[0] for s in systems])
    Qb = block_diag([s[1] for s in systems])
    mb = torch.cat([s[2] for s in systems])
    bb = torch.cat([s[3] for s in systems]).contiguous()
    N = Kb.nrow
    op = SquaredLaplacianOperator(Kb, mb, torch.arange(N, dtype=torch.int32, device=dev),
                                  mass_weight=ALPHA)
    multi = MultiSystemSolver(op, FSAI(Qb, max_row_size=8), sizes)
    xb = torch.zeros_like(bb)

    def run_multi():
        xb.zero_()
        nit, _, _ = multi.run(bb, xb, tol=tol, maxiter=100000)
        return nit

    run_multi()
    t_multi, its_multi = timed(run_multi)
    # The same systems each on its own thread-block cluster, one launch, no
    # concatenation (multi.ClusterSolver).
    from warp_preconditioners_gb300.multi import ClusterSolver

    csolver = ClusterSolver([(s[0], s[1].M) for s in solo])
    cbs = [s[2] for s in solo]
    cxs = [torch.zeros_like(b) for b in cbs]

    def run_cluster():
        for x in cxs:
            x.zero_()
        nit, _, _ = csolver.run(cbs, cxs, tol=tol, maxiter=100000)
        return nit

    run_cluster()
    t_cluster, its_cluster = timed(run_cluster)
    its_solo = [int(i.item()) for i in its_solo]
    its_multi = [int(i) for i in its_multi.cpu().tolist()]
    its_cluster = [int(i) for i in its_cluster.cpu().tolist()]
    S = len(sizes)
    return {"workload": (f"{S} biharmonic smoothing systems on tet cubes of sides "
                         f"{min(sides)}..{max(sides)} ({min(sizes)}..{max(sizes)} unknowns, "
                         f"{N} in all), FSAI w8, CG to {tol:g}, first right-hand side"),
            "one_at_a_time_ms": t_solo, "one_launch_ms": t_multi,
            "one_at_a_time_solves_per_s": S * 1e3 / t_solo,
            "one_launch_solves_per_s": S * 1e3 / t_multi, "speedup": t_solo / t_multi,
            "cluster_per_system_ms": t_cluster,
            "cluster_per_system_solves_per_s": S * 1e3 / t_cluster,
            "cluster_speedup": t_solo / t_cluster,
            "iterations_one_at_a_time": its_solo, "iterations_one_launch": its_multi,
            "iterations_cluster_per_system": its_cluster}


def measure_batched_rhs4(args, prob, Q, K, mass, dev, ms_per_step):
    """The same step (setup + the four right-hand sides) with the four solved
    together by the batched float64 PCG (rows packed 8 per warp, 4 lanes per
    row; matrix bytes read once per iteration for all four), against the
    drop-in one-at-a-time step timed above.  CUDA events, median of 3."""
    import torch

    from warp_preconditioners_gb300 import FSAI, batched

    B = torch.as_tensor(prob["rhs"].T.copy(), device=dev).contiguous()  # [n, 4]
    X = torch.zeros_like(B)

    def step():
        pre = FSAI(Q, max_row_size=args.width, max_step_size=args.step_size, kap_tolerance=1e-3)
        bs = batched.BatchedSolver(K, mass, ALPHA, pre)
        X.zero_()
        return bs.solve(B, X, tol=args.rtol, maxiter=100000)

    step()
    times = []
    for _ in range(3):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        nit, _ = step()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    t = statistics.median(times)
    qh = prob["Q"]
    x = X.cpu().numpy()
    berr = max(float(np.max(np.abs(prob["rhs"][k] - qh @ x[:, k])
                            / (abs(qh) @ np.abs(x[:, k]) + np.abs(prob["rhs"][k]))))
               for k in range(4))
    return {"solver": "one batched float64 PCG for the 4 right-hand sides (FSAI w8)",
            "ms_per_step": t, "solves_per_s": 4000.0 / t,
            "speedup_vs_drop_in": ms_per_step / t,
            "iterations": [int(i) for i in nit.cpu()], "backward_error_max": berr}


def measure_assembly(prob, dev):
    """Q = alpha M + K M^-1 K: the reference's host SciPy product (the
    workload's untimed assembly) against sparse.spgemm on the device (same
    summation order; CUDA-event median of 3, inputs resident)."""
    import torch

    from warp_preconditioners_gb300 import from_scipy, problems, sparse

    t = time.perf_counter()
    host = problems.biharmonic(prob["K"], prob["mass"], ALPHA)
    host_ms = (time.perf_counter() - t) * 1e3
    K = from_scipy(prob["K"], dev)
    m = torch.as_tensor(prob["mass"], device=dev)
    d, e = 1.0 / m, ALPHA * m
    times = []
    for _ in range(3):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        Q = sparse.spgemm(K, K, col_scale=d, add_diag=e)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    vals = Q.values.cpu().numpy()
    same = (Q.nnz == host.nnz and np.array_equal(Q.columns.cpu().numpy(), host.indices))
    return {"host_scipy_ms": host_ms, "device_ms": statistics.median(times), "nnz": Q.nnz,
            "same_pattern": bool(same),
            "max_rel_diff": float(np.max(np.abs(vals - host.data) / np.abs(host.data)))
            if same else None}


def measure_lifted_gmres(args, prob, dev, restart=31, maxiter=30000):
    """The reference's lifted-gmres method (benchmarks/dragon.py:99-118) on the
    smoothing system: Q / alpha = M + tau K M^-1 K with tau = 1/alpha, lifted
    to the interleaved 2x2-block first-order system, GMRES(restart)
    preconditioned by FSAI of H = M + sqrt(tau) K applied to both components,
    first right-hand side (divided by alpha), to the bench's tolerance.
    CUDA-event timing; the accuracy is the componentwise backward error of the
    extracted u on Q."""
    import torch

    from warp_preconditioners_gb300 import BiharmonicSystem, from_scipy, linear

    K = from_scipy(prob["K"], dev)
    mass = torch.as_tensor(prob["mass"], device=dev)
    tau = 1.0 / ALPHA

    def ev():
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        return e

    torch.cuda.synchronize()
    e0 = ev()
    system = BiharmonicSystem(K, mass, tau)
    pre = system.preconditioner(max_row_size=args.width, kap_tolerance=1e-3,
                                max_step_size=args.step_size)
    e1 = ev()
    torch.cuda.synchronize()
    b0 = torch.as_tensor(prob["rhs"][0] / ALPHA, device=dev)
    b = system.rhs(b0)
    x = torch.zeros_like(b)
    solver = linear.GmresSolver(system.matrix, pre, restart=restart)
    solver.run(b, x, args.rtol, 0.0, 5)  # capture the graph
    x.zero_()
    torch.cuda.synchronize()
    e2 = ev()
    nit, res, target = solver.run(b, x, args.rtol, 0.0, maxiter)
    e3 = ev()
    torch.cuda.synchronize()
    u = system.solution(x).cpu().numpy()
    Q = prob["Q"]
    rhs = prob["rhs"][0]
    berr = float(np.max(np.abs(rhs - Q @ u) / (abs(Q) @ np.abs(u) + np.abs(rhs))))
    return {"method": f"lifted 2x2-block system, GMRES({restart}) + FSAI w{args.width} of "
                      f"M + sqrt(tau) K on both components, tau = 1/alpha",
            "setup_ms": e0.elapsed_time(e1), "solve_ms": e2.elapsed_time(e3),
            "iterations": int(nit.item()), "residual": float(res.item()),
            "target": float(target.item()), "backward_error": berr}


def run_gmres_steps(args, dev):
    """Arnoldi-step cost of GMRES(31) on the lifted 2x2-block biharmonic
    system of the --side tet cube (tau = 1e4, FSAI w8 of H = M + sqrt(tau) K
    on both components): --gmres-steps steps from x = 0 on a unit right-hand
    side with an unreachable tolerance, so every step runs."""
    import torch

    from warp_preconditioners_gb300 import BiharmonicSystem, from_scipy, linear, problems

    torch.cuda.set_device(dev)
    _, _, K, mass = problems.tet_cube(args.side)
    system = BiharmonicSystem(from_scipy(K, dev), torch.as_tensor(mass, device=dev), 1e4)
    pre = system.preconditioner(max_row_size=args.width, kap_tolerance=1e-3)
    b = system.rhs(torch.ones(K.shape[0], dtype=torch.float64, device=dev))
    x = torch.zeros_like(b)
    solver = linear.GmresSolver(system.matrix, pre, restart=31,
                                use_cuda_graph=not args.host_loop)
    solver.run(b, x, 1e-14, 0.0, 5)
    x.zero_()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    nit, res, _ = solver.run(b, x, 1e-14, 0.0, args.gmres_steps)
    e1.record()
    torch.cuda.synchronize()
    steps = int(nit.item())
    return {"config": {"workload": f"lifted biharmonic, {args.side}^3 tet cube "
                                   f"({2 * K.shape[0]} unknowns), GMRES(31) + FSAI w{args.width}",
                       "loop": "host" if args.host_loop else "graph"},
            "metric": "ms per Arnoldi step", "steps": steps,
            "ms_per_step": e0.elapsed_time(e1) / max(steps, 1)}


def run_c1(args, dev):
    """The reference's CPU-runnable case: 64 x 64 interior 5-point Dirichlet
    Laplacian (4,096 unknowns, unscaled stencil), U[-1,1] right-hand side
    (seed 0), FSAI w8 step 1 kap 1e-3, CG to 1e-8 from x = 0.  GPU setup and
    solve are CUDA-event medians of 5 (the solve is one graph launch); the
    oracle (CPU restatement, all host threads) runs the same setup and solve
    as the CPU baseline, and its iteration count and solution are the
    parity check."""
    import torch

    from warp_preconditioners_gb300 import FSAI, from_scipy, linear, problems

    torch.cuda.set_device(dev)
    a = problems.laplacian_2d(64)
    b_np = problems.uniform_rhs(a.shape[0], 0)
    A = from_scipy(a, dev)
    b = torch.as_tensor(b_np, device=dev)
    x = torch.zeros_like(b)

    def timed(fn, reps=5):
        out = []
        for _ in range(reps):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r = fn()
            e1.record()
            torch.cuda.synchronize()
            out.append(e0.elapsed_time(e1))
        return statistics.median(out), r

    setup_ms, pre = timed(lambda: FSAI(A, max_row_size=8, max_step_size=1, kap_tolerance=1e-3))
    solver = linear.Solver("cg", A, pre)

    def solve():
        x.zero_()
        return solver.run(b, x, tol=args.rtol, maxiter=10000)

    solve()
    solve_ms, (nit, rr, atol_sq) = timed(solve)
    out = {"config": {"workload": "C1: 64x64 5-point Dirichlet Laplacian (4,096 unknowns), "
                                  "FSAI w8 step 1 kap 1e-3, CG to %g, x0 = 0" % args.rtol},
           "setup_ms": setup_ms, "solve_ms": solve_ms, "iterations": int(nit.item()),
           "converged": bool(rr.item() <= atol_sq.item()),
           "true_relres": float(np.linalg.norm(b_np - a @ x.cpu().numpy()) / np.linalg.norm(b_np))}
    if not args.no_cpu_baseline:
        from oracle import oracle

        c = oracle.CSR(a.indptr, a.indices, a.data)
        t0 = time.perf_counter()
        g, gt, _ = oracle.fsai(c, width=8, step=1, tol=1e-3)
        t1 = time.perf_counter()
        x_or, it_or, _, _ = oracle.krylov("cg", oracle.Operator.csr(c), b_np,
                                          M=oracle.Operator.fsai(g, gt), tol=args.rtol,
                                          maxiter=10000)
        t2 = time.perf_counter()
        out["cpu_baseline"] = {"setup_ms": (t1 - t0) * 1e3, "solve_ms": (t2 - t1) * 1e3,
                               "iterations": it_or, "cores": oracle.num_threads(),
                               "kind": "port",
                               "max_rel_diff_x": float(np.max(np.abs(x.cpu().numpy() - x_or))
                                                       / np.max(np.abs(x_or)))}
    return out


def run_c2_sweep(args, dev):
    """The smoothing system's FSAI variants: (width, step) in {8, 48} x {1, 2}
    with kap 1e-3, and the tuned kap 3e-3 with a float32 factor, under CG and
    CR; first right-hand side, to the bench tolerance.  Setup (FSAI on Q) and
    solve are CUDA-event medians of 3; accuracy is the componentwise backward
    error on Q."""
    import torch

    from warp_preconditioners_gb300 import FSAI, SquaredLaplacianOperator, from_scipy, linear

    torch.cuda.set_device(dev)
    prob = build_problem(args.side)
    n = prob["n"]
    Q = from_scipy(prob["Q"], dev)
    K = from_scipy(prob["K"], dev)
    mass = torch.as_tensor(prob["mass"], device=dev)
    free = torch.arange(n, dtype=torch.int32, device=dev)
    op = SquaredLaplacianOperator(K, mass, free, mass_weight=ALPHA)
    b = torch.as_tensor(prob["rhs"][0], device=dev).contiguous()
    qh = prob["Q"]
    absq = abs(qh)

    def ev(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), out

    variants = [(8, 1, 1e-3, None), (8, 2, 1e-3, None), (48, 1, 1e-3, None),
                (48, 2, 1e-3, None), (8, 1, 3e-3, torch.float32)]
    rows = {}
    for w, step, kap, fdt in variants:
        make = lambda: FSAI(Q, max_row_size=w, max_step_size=step, kap_tolerance=kap,
                            factor_dtype=fdt)
        make()
        setups = []
        for _ in range(3):
            t, pre = ev(make)
            setups.append(t)
        for method in ("cg", "cr"):
            solver = linear.Solver(method, op, pre)
            x = torch.zeros(n, dtype=torch.float64, device=dev)
            solver.run(b, x, tol=args.rtol, maxiter=100000)
            times = []
            for _ in range(3):
                x.zero_()
                t, (nit, rr, at) = ev(lambda: solver.run(b, x, tol=args.rtol, maxiter=100000))
                times.append(t)
            u = x.cpu().numpy()
            rhs = prob["rhs"][0]
            berr = float(np.max(np.abs(rhs - qh @ u) / (absq @ np.abs(u) + np.abs(rhs))))
            name = f"w{w}_step{step}_kap{kap:g}" + ("_f32" if fdt is not None else "") + f"/{method}"
            rows[name] = {"setup_ms": statistics.median(setups),
                          "solve_ms": statistics.median(times),
                          "iterations": int(nit.item()), "converged": bool(rr.item() <= at.item()),
                          "factor_nnz": pre.G.nnz, "backward_error": berr}
    return {"config": {"workload": f"biharmonic smoothing, {args.side}^3 tet cube, first RHS, "
                                   f"CG/CR to {args.rtol:g}, FSAI variants"},
            "metric": "setup + solve ms per FSAI variant and solver", "results": rows}


def run_c3(args, dev, maxiter=20000):
    """K (x) C block coupling: K = 7-point Dirichlet Laplacian on an n^3 grid,
    C = R diag(1, 1, 1e-6) R^T with a seeded rotation, 3x3 blocks, float64;
    every preconditioner of the reference's block benchmark
    (benchmarks/block_challenge.py:249-261) under CG and CR to 1e-8, from
    zero, on a U[-1,1] right-hand side.  Setup and solve are timed
    separately with CUDA events (medians of 3)."""
    import torch

    from warp_preconditioners_gb300 import (BlockILU0, BlockJacobi, BsrBlockFSAI, FSAI, problems,
                                            from_scipy, linear)

    torch.cuda.set_device(dev)
    bsr, c = problems.kron_coupling(args.c3_grid, 1e-6, seed=0)
    bsr.sort_indices()
    A = from_scipy(bsr.tocsr(), dev, torch.float64, (3, 3))
    n = bsr.shape[0]
    b_np = problems.uniform_rhs(n, 0)
    b = torch.as_tensor(b_np, device=dev)
    makers = {
        "scalar_jacobi": lambda: linear.preconditioner(A, "diag"),
        "block_jacobi": lambda: BlockJacobi(A, pivot_tolerance=1e-15),
        "fsai_w8": lambda: FSAI(A, max_row_size=8, kap_tolerance=0.003,
                                factor_dtype=torch.float32),
        "block_fsai_2": lambda: BsrBlockFSAI(A, max_blocks=2, factor_dtype=torch.float32),
        "block_fsai_4": lambda: BsrBlockFSAI(A, max_blocks=4, factor_dtype=torch.float32),
        "block_ilu0_3_3": lambda: BlockILU0(A, factor_sweeps=3, solve_sweeps=3,
                                            pivot_tolerance=1e-15),
    }

    def ev_time(fn):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        out = fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), out

    rows = {}
    for name, make in makers.items():
        make()
        setups = []
        for _ in range(3):
            t, pre = ev_time(make)
            setups.append(t)
        for method in ("cg", "cr"):
            solver = linear.Solver(method, A, pre)
            x = torch.zeros(n, dtype=torch.float64, device=dev)
            solver.run(b, x, tol=args.rtol, maxiter=maxiter)
            times = []
            for _ in range(3):
                x.zero_()
                t, (nit, rr, at) = ev_time(lambda: solver.run(b, x, tol=args.rtol,
                                                              maxiter=maxiter))
                times.append(t)
            sol = x.cpu().numpy()
            rel = float(np.linalg.norm(b_np - bsr @ sol) / np.linalg.norm(b_np))
            it = int(nit.item())
            rows[f"{name}/{method}"] = {
                "setup_ms": statistics.median(setups), "solve_ms": statistics.median(times),
                "total_ms": statistics.median(setups) + statistics.median(times),
                "iterations": it, "converged": bool(rr.item() <= at.item()),
                "true_relres": rel}
    return {"config": {"workload": f"K (x) C, {args.c3_grid}^3 7-point Laplacian, C = R diag(1,1,"
                                   f"1e-6) R^T, 3x3 BSR float64, {n} unknowns, CG/CR to "
                                   f"{args.rtol:g} (max {maxiter} iterations), U[-1,1] RHS"},
            "metric": "setup+solve ms per preconditioner and solver", "results": rows}


def run_c5(args, dev):
    """Serving stream: the first --c5-requests requests of the seed-0 stream of
    2,000 (Laplacian or tet-cube biharmonic, n log-uniform on [5e3, 5e5],
    1-8 U[-1,1] right-hand sides, Poisson arrivals at --c5-rate per second),
    CG + FSAI w8 to 1e-8 relative residual, systems resident under the HBM
    budget.  Served with continuous batching into slots, then replayed on the
    plain one-at-a-time float64 path; latency is from the scheduled arrival
    to x back in host memory.  Each arm also replays the same requests all
    arriving at once ("burst"): its solves/s is the arm's capacity."""
    import torch

    from warp_preconditioners_gb300 import serve

    torch.cuda.set_device(dev)
    full = serve.request_stream(2000, args.c5_rate, seed=0, n_min=args.c5_nmin,
                                n_max=args.c5_nmax)
    stream = full[:args.c5_requests]
    keys = list(dict.fromkeys(r.key for r in stream))
    cat = serve.Catalog()
    t0 = time.perf_counter()
    cat.prebuild(keys, threads=min(16, os.cpu_count() or 4))
    assembly_s = time.perf_counter() - t0

    budget = args.c5_budget_gb * 1e9
    ex = serve.GpuExecutor(cat, slots=args.c5_slots, tol=args.rtol, device=dev)
    srv = serve.Server(ex, budget_bytes=budget)
    t0 = time.perf_counter()
    srv.prepare(keys)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    burst = [serve.Request(r.rid, r.kind, r.side, r.k, 0.0, r.seed) for r in stream]
    keep = lambda r: r.rid % 10 == 0
    with ClockSampler(dev.index or 0) as clk:
        served = srv.run(stream, keep=keep)
        served_burst = srv.run(burst, keep=lambda r: False)
    clocks = clk.summary()
    out = {"served": serve.summarize(served), "served_burst": serve.summarize(served_burst)}

    # Every tenth request, on the host (untimed): relative residual
    # |b - A x| / |b| and componentwise backward error
    # max_i |b - A x|_i / (|A| |x| + |b|)_i.  For the alpha = 1e-4 biharmonic
    # systems the first is dominated by cancellation in forming b - A x
    # (|A| |x| >> |b|); the second is the accuracy measure.
    assembled = {}

    def sample_accuracy(reqs, results):
        acc = {kind: {"rel": [], "berr": []} for kind in serve.KINDS}
        nonfinite = 0
        for req, r in zip(reqs, results):
            if r.ok and r.x is not None:
                h = cat.get(req.key)
                if req.key not in assembled:  # host assembly for the check only
                    assembled[req.key] = h.assembled()
                A = assembled[req.key]
                b, x = serve.request_rhs(req).numpy(), r.x.numpy()
                if not np.isfinite(x).all():
                    nonfinite += 1
                    continue
                res = b - A @ x
                acc[h.kind]["rel"].append(float((np.linalg.norm(res, axis=0)
                                                 / np.linalg.norm(b, axis=0)).max()))
                den = abs(A) @ np.abs(x) + np.abs(b)
                acc[h.kind]["berr"].append(float((np.abs(res) / den).max()))
        summary = {kind: {"requests": len(a["rel"]),
                          "relres_max": max(a["rel"]) if a["rel"] else None,
                          "backward_error_max": max(a["berr"]) if a["berr"] else None}
                   for kind, a in acc.items()}
        summary["checked_requests"] = sum(len(a["rel"]) for a in acc.values()) + nonfinite
        summary["nonfinite_solutions"] = nonfinite
        return summary

    sampled = sample_accuracy(stream, served)
    out["served"]["checked_requests"] = sampled.pop("checked_requests")
    out["served"]["nonfinite_solutions"] = sampled.pop("nonfinite_solutions")
    out["served"]["accuracy_sampled"] = sampled

    if args.c5_merge:
        mex = serve.GpuExecutor(cat, slots=args.c5_slots, tol=args.rtol, device=dev,
                                merge_rhs=args.c5_merge)
        msrv = serve.Server(mex, budget_bytes=budget)
        t0 = time.perf_counter()
        msrv.prepare(keys)
        torch.cuda.synchronize()
        out["served_merged_setup_s"] = time.perf_counter() - t0
        out["served_merged"] = serve.summarize(msrv.run(stream, keep=lambda r: False))
        out["served_merged_burst"] = serve.summarize(msrv.run(burst, keep=lambda r: False))
        del msrv, mex
    if args.c5_cluster_small:
        bex = serve.GpuExecutor(cat, slots=args.c5_slots, tol=args.rtol, device=dev,
                                cluster_rhs=True)
        bsrv = serve.Server(bex, budget_bytes=budget)
        bsrv.prepare(keys)
        torch.cuda.synchronize()
        out["served_cluster_small"] = serve.summarize(bsrv.run(stream, keep=lambda r: False))
        out["served_cluster_small_burst"] = serve.summarize(bsrv.run(burst, keep=lambda r: False))
        del bsrv, bex
    if args.c5_wide_from:
        wex = serve.GpuExecutor(cat, slots=args.c5_slots, tol=args.rtol, device=dev,
                                wide_from=args.c5_wide_from, wide_step=args.c5_wide_step)
        wsrv = serve.Server(wex, budget_bytes=budget)
        t0 = time.perf_counter()
        wsrv.prepare(keys)
        torch.cuda.synchronize()
        out["served_wide_setup_s"] = time.perf_counter() - t0
        wide_res = wsrv.run(stream, keep=keep)
        out["served_wide"] = serve.summarize(wide_res)
        out["served_wide"]["accuracy_sampled"] = sample_accuracy(stream, wide_res)
        out["served_wide_burst"] = serve.summarize(wsrv.run(burst, keep=lambda r: False))
        del wsrv, wex
    if not args.c5_no_sequential:
        seq_ex = serve.GpuExecutor(cat, sequential=True, tol=args.rtol, device=dev)
        seq = serve.Server(seq_ex, budget_bytes=budget)
        seq.resident, seq.used, seq.peak = srv.resident, srv.used, srv.peak  # same systems
        out["sequential"] = serve.summarize(seq.run(stream, keep=lambda r: False))
        out["sequential_burst"] = serve.summarize(seq.run(burst, keep=lambda r: False))
        s, q = out["served"], out["sequential"]
        sb, qb = out["served_burst"], out["sequential_burst"]
        out["speedup"] = {"capacity_solves_per_s": sb["solves_per_s"] / qb["solves_per_s"],
                          "p50": q["p50_ms"] / s["p50_ms"], "p99": q["p99_ms"] / s["p99_ms"]}
        if args.c5_wide_from:
            mb, m = out["served_wide_burst"], out["served_wide"]
            out["speedup_wide"] = {
                "capacity_solves_per_s": mb["solves_per_s"] / qb["solves_per_s"],
                "p50": q["p50_ms"] / m["p50_ms"], "p99": q["p99_ms"] / m["p99_ms"]}
        if args.c5_cluster_small:
            mb, m = out["served_cluster_small_burst"], out["served_cluster_small"]
            out["speedup_cluster_small"] = {
                "capacity_solves_per_s": mb["solves_per_s"] / qb["solves_per_s"],
                "p50": q["p50_ms"] / m["p50_ms"], "p99": q["p99_ms"] / m["p99_ms"]}
        if args.c5_merge:
            mb, m = out["served_merged_burst"], out["served_merged"]
            out["speedup_merged"] = {
                "capacity_solves_per_s": mb["solves_per_s"] / qb["solves_per_s"],
                "p50": q["p50_ms"] / m["p50_ms"], "p99": q["p99_ms"] / m["p99_ms"]}
    kinds = collections.Counter(r.kind for r in stream)
    return {
        "metric": "serving p50/p99 latency (ms) and solves/s at 1e-8 relative residual",
        "unit": "ms, solves/s", "higher_is_better": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"serving stream: first {len(stream)} of 2,000 seeded requests "
                               f"(seed 0), Poisson {args.c5_rate:g}/s, n log-uniform "
                               f"[{args.c5_nmin:g}, {args.c5_nmax:g}], 1-8 U[-1,1] RHS, "
                               f"{dict(kinds)}; CG + FSAI w8 to {args.rtol:g}",
                   "slots": ex.slots, "budget_gb": args.c5_budget_gb,
                   "systems": len(keys)},
        "host_assembly_s": assembly_s, "device_setup_s": setup_s,
        "resident_gb": srv.used / 1e9, "resident_peak_gb": srv.peak / 1e9,
        "server_stats": srv.stats, "clocks": clocks, **out}


def launch_count(iters, width=8):
    """Kernels of ours launched per timed step, times steps (structure of the code):
    setup = sqlap (index, mass, gather, boundary map, 3 x SELL build of 2 kernels + scan)
    + FSAI (diag, prep, build by rounds: init, 2 per round x (width - 1), finish;
    scan 3, pack, transpose 6, 2 x SELL build 3) ; solve = init 7 + 6 per CG iteration."""
    setup = 4 + 3 * 3 + (2 + 2 + 2 * (width - 1)) + 3 + 1 + 6 + 2 * 3
    return sum(setup + sum(7 + 6 * i for i in step) for step in iters)


def _graph_time(fns, reps, dev):
    """Seconds per call of the calls in `fns` (cycled), `reps` of them
    replayed from one CUDA graph, CUDA events around a warm replay."""
    import torch

    side = torch.cuda.Stream(dev)
    side.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(side):
        for fn in fns:
            fn()
    torch.cuda.current_stream(dev).wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        for r in range(reps):
            fns[r % len(fns)]()
    graph.replay()
    torch.cuda.synchronize()
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    s.record()
    graph.replay()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps / 1e3


def measure_applies(pre, make_pre, K, mass, free, n, dev, copies=5, make_low=None):
    """Live CUDA-event timing of the two applies on the step's data,
    algorithmic bytes over the time (GB/s), two ways:

    * ``resident``: 50 back-to-back applies of one operator replayed from one
      graph; the FSAI factor (66 MB) stays in L2 between them, so this is the
      apply's issue-bound rate, not an HBM figure;
    * ``hbm``: 50 applies cycling over `copies` independent operators and
      vectors (more than twice the 129 MB L2 in total), so every apply reads
      its matrices from HBM.  Reuse inside one apply (the factored operator
      reads its one copy of L twice) still counts, as it does in a solve.

    ``fsai_apply_bf16_f32``: the same FSAI factor stored in bfloat16 and
    applied in float32 behind the float64 interface (x read as float64, the
    intermediate G x as float32, z written as float64); no FP64 arithmetic.
    """
    import torch

    from warp_preconditioners_gb300 import SquaredLaplacianOperator

    ops = [SquaredLaplacianOperator(K, mass, free, mass_weight=ALPHA) for _ in range(copies)]
    pres = [pre] + [make_pre() for _ in range(copies - 1)]
    xs = [torch.randn(n, dtype=torch.float64, device=dev) for _ in range(copies)]
    zs = [torch.empty_like(x) for x in xs]
    out = {}
    reps = 50
    fsai_bytes = (pre.G.nnz + pre.GT.nnz) * 12 + 2 * 4 * (n + 1) + 4 * n * 8
    op_bytes = 2 * (K.nnz * 12 + 4 * (n + 1)) + 6 * n * 8

    def fsai_call(c):
        return lambda: pres[c].matvec(xs[c], xs[c], zs[c], 1.0, 0.0)

    def op_call(c):
        return lambda: ops[c].matvec(xs[c], xs[c], zs[c], 1.0, 0.0)

    for name, make, nbytes, footprint in (
        ("fsai_apply", fsai_call, fsai_bytes, fsai_bytes),
        ("factored_operator_apply", op_call, op_bytes, K.nnz * 12 + 6 * n * 8),
    ):
        t_res = _graph_time([make(0)], reps, dev)
        t_hbm = _graph_time([make(c) for c in range(copies)], reps, dev)
        out[name] = {"us": t_res * 1e6, "gbps": nbytes / t_res / 1e9, "bytes": nbytes,
                     "hbm": {"us": t_hbm * 1e6, "gbps": nbytes / t_hbm / 1e9,
                             "copies": copies, "rotated_bytes": copies * footprint}}
    if make_low is not None:
        lows = [make_low() for _ in range(copies)]
        low = lows[0]
        nbytes = (low.G.nnz + low.GT.nnz) * 6 + 2 * 4 * (n + 1) + n * (8 + 4 + 4 + 8)
        calls = [(lambda c: lambda: lows[c].matvec(xs[c], xs[c], zs[c], 1.0, 0.0))(c)
                 for c in range(copies)]
        t_res = _graph_time(calls[:1], reps, dev)
        t_hbm = _graph_time(calls, reps, dev)
        out["fsai_apply_bf16_f32"] = {
            "us": t_res * 1e6, "gbps": nbytes / t_res / 1e9, "bytes": nbytes,
            "hbm": {"us": t_hbm * 1e6, "gbps": nbytes / t_hbm / 1e9, "copies": copies,
                    "rotated_bytes": copies * nbytes}}
    return out


def read_traffic():
    """Measured DRAM bytes per PCG iteration from the committed ncu summary, if any."""
    p = ROOT / "profiles" / "pcg_iteration_traffic.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("dram_bytes_per_iteration:"):
            return float(line.split(":")[1])
    return None


def run_e2e(args, prob, dev, one_step, world, dist):
    """Same metric from pinned host buffers through the public API."""
    import torch

    from warp_preconditioners_gb300.sparse import BsrMatrix

    Qh, Kh = prob["Q"], prob["K"]

    def pinned(a, dtype=None):
        t = torch.as_tensor(np.ascontiguousarray(a))
        if dtype is not None:
            t = t.to(dtype)
        return t.pin_memory()

    host = {
        "q_off": pinned(Qh.indptr.astype(np.int32)), "q_col": pinned(Qh.indices.astype(np.int32)),
        "q_val": pinned(Qh.data), "k_off": pinned(Kh.indptr.astype(np.int32)),
        "k_col": pinned(Kh.indices.astype(np.int32)), "k_val": pinned(Kh.data),
        "mass": pinned(prob["mass"]), "rhs": pinned(prob["rhs"]),
    }
    out_host = torch.empty((4, prob["n"]), dtype=torch.float64).pin_memory()
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    d2h = out_host.numel() * out_host.element_size()

    def step():
        d = {k: v.to(dev, non_blocking=True) for k, v in host.items()}
        Qm = BsrMatrix(Qh.shape[0], Qh.shape[1], (1, 1), d["q_off"], d["q_col"], d["q_val"])
        Km = BsrMatrix(Kh.shape[0], Kh.shape[1], (1, 1), d["k_off"], d["k_col"], d["k_val"])
        xs = torch.empty((4, prob["n"]), dtype=torch.float64, device=dev)
        one_step(Qm, Km, d["mass"], d["rhs"], xs)
        out_host.copy_(xs, non_blocking=True)

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(args.steps):
        step()
    e.record()
    torch.cuda.synchronize()
    value, ms = replica_aggregate(s.elapsed_time(e), 4.0 * args.steps, dist, dev)
    return {"value": value, "unit": "solves/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": ms / args.steps}


if __name__ == "__main__":
    main()
