"""Generate the known-answer fixtures in tests/golden/ (run from the repo root).

The reference ships no stored vectors; its tests compute known answers with
dense NumPy.  This script restates those computations independently of the
oracle and of the CUDA path and stores inputs plus expected outputs:

* fsai_greedy.npz   tests/test_fsai.py:125-169 — independent greedy support
                    search on the rng(193) 18 x 18 matrix, for kap tolerances
                    {0, 0.003, 0.1} and step sizes {1, 3}.
* fsai_path.npz     tests/test_fsai.py:189-203 — path graph, width 8: supports
                    arange(max(0, i-7), i+1) and exact local-solve values.
* fsai_full.npz     tests/test_fsai.py:36-51, :206-213 — full supports give
                    G^T G = A^-1 (rng(7) 8 x 8 and the n = 32 tridiagonal).
* fsai_scaled.npz   tests/test_fsai.py:73-90 — per-row local solves on a
                    severely scaled tridiagonal (rng(18)), width 5.
* ilu0_recurrence.npz tests/test_indefinite.py:148-177 — block ILU(0) factors
                    from the sequential recurrence (rng(83), 2 x 2 blocks).
* sqlap.npz         tests/test_squared_laplacian.py:12-63 — the reduced
                    operator (L M^-1 L + w M)[free, free] and the eliminated
                    right-hand side (rng(27)).
* block_jacobi_spectrum.npz tests/test_block_challenge.py:47-60 — K (x) C
                    with block Jacobi has spectrum {1/2, 5/6, 7/6, 3/2}.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import scipy.sparse as ss

OUT = Path(__file__).resolve().parent


def greedy_fsai(a, width, step, tolerance):
    """Dense restatement of the greedy search in tests/test_fsai.py:143-168."""
    n = len(a)
    equilibrated = a / np.sqrt(np.diag(a)[:, None] * np.diag(a)[None, :])
    g = np.zeros_like(a)
    for i in range(n):
        support = [i]
        z = np.ones(1)
        while len(support) < width:
            frontier = sorted(set(np.flatnonzero(np.any(a[support] != 0, axis=0))) - set(support))
            frontier = [c for c in frontier if c < i]
            if not frontier:
                break
            scores = [abs(equilibrated[c, support] @ z) for c in frontier]
            selected = sorted(zip(scores, frontier), key=lambda item: (-item[0], item[1]))
            selected = [c for score, c in selected if score > 0][: min(step, width - len(support))]
            if not selected:
                break
            support.extend(selected)
            old = z[0]
            rhs = np.zeros(len(support))
            rhs[0] = 1
            z = np.linalg.solve(equilibrated[np.ix_(support, support)], rhs)
            if 1 - old / z[0] <= tolerance:
                break
        g[i, support] = z / np.sqrt(z[0] * np.diag(a)[support])
    return g


def fsai_greedy():
    rng = np.random.default_rng(193)
    a = rng.normal(size=(18, 18))
    a[rng.random(a.shape) < 0.65] = 0
    a = a + a.T
    np.fill_diagonal(a, np.sum(np.abs(a), axis=1) + 2)
    scaling = np.geomspace(0.01, 100, 18)
    a *= scaling[:, None] * scaling[None, :]
    out = {"a": a}
    for tol in (0.0, 0.003, 0.1):
        for step in (1, 3):
            out[f"g_tol{tol}_step{step}"] = greedy_fsai(a, 8, step, tol)
    np.savez_compressed(OUT / "fsai_greedy.npz", **out)


def tridiagonal(n, d=3.0):
    return np.diag(np.full(n, d)) + np.diag(-np.ones(n - 1), 1) + np.diag(-np.ones(n - 1), -1)


def fsai_path():
    a = tridiagonal(12)
    g = np.zeros_like(a)
    for i in range(12):
        support = np.arange(max(0, i - 7), i + 1)
        rhs = np.zeros(len(support))
        rhs[-1] = 1
        z = np.linalg.solve(a[np.ix_(support, support)], rhs)
        g[i, support] = z / np.sqrt(z[-1])
    np.savez_compressed(OUT / "fsai_path.npz", a=a, g=g,
                        counts=np.minimum(np.arange(1, 13), 8))


def fsai_full():
    rng = np.random.default_rng(7)
    a = rng.normal(size=(8, 8))
    a = a @ a.T + np.eye(8)
    x = rng.normal(size=8)
    y = rng.normal(size=8)
    b32 = tridiagonal(32)
    np.savez_compressed(OUT / "fsai_full.npz", a8=a, inv8=np.linalg.inv(a), x8=x, y8=y,
                        a32=b32, inv32=np.linalg.inv(b32))


def fsai_scaled():
    a = tridiagonal(20, 4.0)
    scale = np.geomspace(1e-4, 1e4, 20)
    a = scale[:, None] * a * scale[None, :]
    np.savez_compressed(OUT / "fsai_scaled.npz", a=a)


def ilu0_recurrence():
    rng = np.random.default_rng(83)
    n, size = 9, 2
    blocks = {}
    for i in range(n):
        for j in range(n):
            if i == j:
                blocks[i, j] = np.diag([3.0, -2.0])
            elif abs(i - j) == 1 or (i + j) % 5 == 0:
                blocks[i, j] = rng.normal(size=(size, size)) * 0.08
    expected = {key: value.copy() for key, value in blocks.items()}
    for i in range(n):
        for j in sorted(j for row, j in blocks if row == i):
            value = blocks[i, j].copy()
            for k in range(min(i, j)):
                if (i, k) in expected and (k, j) in expected:
                    value -= expected[i, k] @ expected[k, j]
            expected[i, j] = value @ np.linalg.inv(expected[j, j]) if j < i else value
    a = np.zeros((size * n, size * n))
    for (i, j), value in blocks.items():
        a[size * i: size * (i + 1), size * j: size * (j + 1)] = value
    keys = sorted(blocks)
    np.savez_compressed(OUT / "ilu0_recurrence.npz", a=a,
                        rows=np.array([k[0] for k in keys]), cols=np.array([k[1] for k in keys]),
                        factors=np.stack([expected[k] for k in keys]))


def sqlap():
    rng = np.random.default_rng(27)
    n = 67
    lap = ss.diags([-np.ones(n - 1), np.r_[1.0, np.full(n - 2, 2.0), 1.0], -np.ones(n - 1)],
                   [-1, 0, 1]).tocsr()
    mass = rng.uniform(0.4, 2, size=n)
    free = rng.permutation(np.arange(3, n - 4)).astype(np.int32)
    out = {"lap": lap.toarray(), "mass": mass, "free": free}
    for w in (0.0, 0.15):
        q = (lap @ ss.diags(1 / mass) @ lap + w * ss.diags(mass)).toarray()
        out[f"reduced_w{w}"] = q[np.ix_(free, free)]
        bc = rng.normal(size=n)
        prescribed = bc.copy()
        prescribed[free] = 0
        out[f"bc_w{w}"] = bc
        out[f"rhs_w{w}"] = -(q @ prescribed)[free]
    np.savez_compressed(OUT / "sqlap.npz", **out)


def block_jacobi_spectrum():
    np.savez_compressed(OUT / "block_jacobi_spectrum.npz",
                        expected=np.repeat([0.5, 5 / 6, 5 / 6, 5 / 6, 7 / 6, 7 / 6, 7 / 6, 1.5], 3))


if __name__ == "__main__":
    fsai_greedy()
    fsai_path()
    fsai_full()
    fsai_scaled()
    ilu0_recurrence()
    sqlap()
    block_jacobi_spectrum()
    print("wrote", sorted(p.name for p in OUT.glob("*.npz")))
