"""Run the reference's own test modules, unmodified, on the Warp emulation.

The reference's tests are parametrised over Warp devices ("cpu" and
"cuda:0"); with the emulation in ``tests/golden/warp_emu`` only "cpu" exists,
so the CUDA parametrisations skip themselves (``wp.is_cuda_available()`` is
False) and every CPU case runs the reference's own kernels and assertions.
Passing them shows that the emulation executes the reference faithfully,
which is what makes ``ref_*.npz`` (tests/golden/make_reference_golden.py)
outputs of the reference itself.

Modules that need Warp internals (``warp._src``: the residual sampler and the
block benchmarks' imports) or are out of the hot path (elasticity, SimJEB,
float16) are not run.  Nothing is written into the reference tree (no
bytecode, no pytest cache).

    python tests/golden/run_reference_tests.py [--write]

``--write`` records the per-module counts in
tests/golden/reference_tests_emulated.txt.
"""

from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REFERENCE = Path(os.environ.get("WARP_PRECONDITIONERS_REF", "/root/reference"))
MODULES = [
    "test_fsai.py",
    "test_sparse_operator.py",
    "test_squared_laplacian.py",
    "test_updates.py",
    "test_indefinite.py",
    "test_fsai_candidates.py",
    "test_biharmonic.py",
]
SUMMARY = HERE / "reference_tests_emulated.txt"


def available() -> bool:
    return (REFERENCE / "warp_preconditioners" / "fsai.py").exists() and all(
        (REFERENCE / "tests" / m).exists() for m in MODULES)


def run(module: str, timeout: float = 900.0) -> dict:
    env = dict(os.environ)
    env["PYTHONDONTWRITEBYTECODE"] = "1"
    env["PYTHONPATH"] = os.pathsep.join([str(HERE / "warp_emu"), str(REFERENCE)])
    cmd = [sys.executable, "-m", "pytest", "-p", "no:cacheprovider", "-q", "-rA",
           "--rootdir", str(REFERENCE / "tests"), str(REFERENCE / "tests" / module)]
    r = subprocess.run(cmd, cwd=str(HERE), env=env, capture_output=True, text=True,
                       timeout=timeout)
    tail = r.stdout.strip().splitlines()[-1] if r.stdout.strip() else ""
    counts = {k: int(v) for v, k in re.findall(r"(\d+) (passed|failed|skipped|error)", tail)}
    passed = sorted(m.group(1) for m in re.finditer(r"^PASSED (\S+)", r.stdout, re.M))
    return {"module": module, "rc": r.returncode, "counts": counts, "passed": passed,
            "tail": tail, "output": r.stdout[-4000:] + r.stderr[-2000:]}


def main(write: bool) -> int:
    if not available():
        print(f"reference tree not found at {REFERENCE}")
        return 2
    results = [run(m) for m in MODULES]
    lines = ["Reference test modules run unmodified on the Warp emulation "
             "(CPU parametrisations; CUDA ones skip themselves).", ""]
    bad = 0
    for res in results:
        c = res["counts"]
        lines.append(f"{res['module']}: {c.get('passed', 0)} passed, {c.get('failed', 0)} "
                     f"failed, {c.get('skipped', 0)} skipped (CUDA)")
        bad += c.get("failed", 0) + c.get("error", 0) + (res["rc"] not in (0,))
    lines.append("")
    for res in results:
        lines.extend("  " + t.split("::", 1)[-1] if "::" in t else "  " + t
                     for t in res["passed"])
    text = "\n".join(lines) + "\n"
    print(text)
    if write:
        SUMMARY.write_text(text)
    return 1 if bad else 0


if __name__ == "__main__":
    sys.exit(main("--write" in sys.argv))
