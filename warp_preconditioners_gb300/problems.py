"""Seeded synthetic inputs for the benchmark configurations (host NumPy/SciPy).

The reference assembles its inputs on the host with SciPy or from mesh files
(benchmarks/synthetic.py:24-30, benchmarks/block_challenge.py:30-117,
visualization/solve_fields.py:220-221); assembly is excluded from timing
there and here.  These generators produce the named shapes:

* ``laplacian_2d(64)``: 5-point Dirichlet Laplacian on a 64 x 64 interior
  grid, unscaled stencil (4 on the diagonal, -1 off it).
* ``tet_cube(70)``: a 70^3-vertex cube on [0, 1]^3, each hex split into six
  tetrahedra along the main diagonal, interior vertices jittered by
  U[-0.2h, 0.2h]^3; P1 cotangent stiffness K (positive semidefinite, zero row
  sums) and barycentric lumped mass M.
* ``biharmonic(K, M, alpha)``: the assembled ``Q = alpha M + K M^-1 K``.
* ``laplacian_3d(64)``: 7-point Dirichlet Laplacian (6 / -1), and
  ``kron_coupling`` = K (x) C with ``C = R diag(1, 1, kappa) R^T``, R a
  seeded Haar rotation, as 3 x 3 blocks.
"""

from __future__ import annotations

import itertools

import numpy as np
import scipy.sparse as ss


def laplacian_1d(n: int) -> ss.csr_matrix:
    return ss.diags([-np.ones(n - 1), 2 * np.ones(n), -np.ones(n - 1)], [-1, 0, 1]).tocsr()


def laplacian_2d(n: int = 64) -> ss.csr_matrix:
    t = laplacian_1d(n)
    a = ss.kronsum(t, t).tocsr()
    a.sort_indices()
    return a


def laplacian_3d(n: int = 64) -> ss.csr_matrix:
    t = laplacian_1d(n)
    a = ss.kronsum(ss.kronsum(t, t), t).tocsr()
    a.sort_indices()
    return a


def uniform_rhs(n: int, seed: int = 0) -> np.ndarray:
    return np.random.default_rng(seed).uniform(-1.0, 1.0, size=n)


def tet_cube(side: int = 70, jitter: float = 0.2, seed: int = 0):
    """Vertices, tets, P1 stiffness K (CSR) and lumped mass of a jittered tet cube."""
    h = 1.0 / (side - 1)
    g = np.arange(side) * h
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    verts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    idx = np.arange(side**3).reshape(side, side, side)  # [z, y, x]
    interior = np.zeros((side, side, side), dtype=bool)
    interior[1:-1, 1:-1, 1:-1] = True
    interior = interior.ravel()
    rng = np.random.default_rng(seed)
    offs = rng.uniform(-jitter * h, jitter * h, size=(int(interior.sum()), 3))
    verts[interior] += offs
    # Cube corners: c[dx, dy, dz] for every cell.
    c = {}
    for dx, dy, dz in itertools.product((0, 1), repeat=3):
        c[(dx, dy, dz)] = idx[dz:side - 1 + dz, dy:side - 1 + dy, dx:side - 1 + dx].ravel()
    tets = []
    for perm in itertools.permutations(range(3)):
        step = [0, 0, 0]
        path = [tuple(step)]
        for axis in perm:
            step[axis] = 1
            path.append(tuple(step))
        tets.append(np.stack([c[p] for p in path], axis=1))
    tets = np.concatenate(tets, axis=0).astype(np.int64)
    p = verts[tets]  # [T, 4, 3]
    e1, e2, e3 = p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]
    # Gradients of barycentric coordinates 1..3 are the rows of the inverse of
    # [e1 e2 e3]: the cross products of the other two edges over the
    # determinant (closed form; batched LAPACK on 3x3 blocks is far slower).
    c23, c31, c12 = np.cross(e2, e3), np.cross(e3, e1), np.cross(e1, e2)
    det = np.einsum("ti,ti->t", e1, c23)
    vol = np.abs(det) / 6.0
    inv_det = (1.0 / det)[:, None]
    g = [None, c23 * inv_det, c31 * inv_det, c12 * inv_det]
    g[0] = -(g[1] + g[2] + g[3])
    local = np.empty((len(tets), 4, 4))
    for a in range(4):
        for b in range(a, 4):
            v = vol * np.einsum("ti,ti->t", g[a], g[b])
            local[:, a, b] = v
            local[:, b, a] = v
    rows = np.repeat(tets, 4, axis=1).ravel()
    cols = np.tile(tets, (1, 4)).ravel()
    nv = side**3
    K = ss.csr_matrix((local.ravel(), (rows, cols)), shape=(nv, nv))
    K.sum_duplicates()
    K.sort_indices()
    K = ((K + K.T) * 0.5).tocsr()  # exact symmetry of the assembled sum
    # Cotangent weights that vanish analytically (right angles on the
    # unjittered boundary faces) come out as +-1e-18 rounding noise; drop
    # them so the sparsity pattern does not depend on the rounding of the
    # host's floating-point library.
    K.data[np.abs(K.data) <= 1e-13 * np.abs(K.data).max()] = 0.0
    K.eliminate_zeros()
    K.sort_indices()
    mass = np.bincount(tets.ravel(), weights=np.repeat(vol / 4.0, 4), minlength=nv)
    return verts, tets, K, mass


def biharmonic(K: ss.csr_matrix, mass: np.ndarray, alpha: float) -> ss.csr_matrix:
    """Assembled Q = alpha M + K M^-1 K (SciPy SpGEMM, as the reference does)."""
    q = (K @ ss.diags(1.0 / mass) @ K + ss.diags(alpha * mass)).tocsr()
    q.sum_duplicates()
    q.sort_indices()
    return q


def smoothing_rhs(verts: np.ndarray, mass: np.ndarray, alpha: float) -> np.ndarray:
    """alpha M f for f = sin(3x) + cos(2y) z + x z, then alpha M {x, y, z}: [4, n]."""
    x, y, z = verts[:, 0], verts[:, 1], verts[:, 2]
    f = np.sin(3 * x) + np.cos(2 * y) * z + x * z
    return np.stack([alpha * mass * f, alpha * mass * x, alpha * mass * y, alpha * mass * z])


def haar_rotation(seed: int = 0) -> np.ndarray:
    q, r = np.linalg.qr(np.random.default_rng(seed).normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))[None, :]
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def kron_coupling(n: int = 64, kappa: float = 1e-6, seed: int = 0):
    """A = K (x) C as 3 x 3 BSR arrays (indptr, indices, blocks) and the scalar CSR."""
    k = laplacian_3d(n)
    r = haar_rotation(seed)
    c = r @ np.diag([1.0, 1.0, kappa]) @ r.T
    blocks = k.data[:, None, None] * c[None, :, :]
    bsr = ss.bsr_matrix((blocks, k.indices, k.indptr), shape=(3 * k.shape[0], 3 * k.shape[1]))
    return bsr, c
