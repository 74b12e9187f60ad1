"""Adaptive, diagonally equilibrated FSAI: P = G^T G (warp_preconditioners/fsai.py).

Setup is one libgbpc call per stage: adaptive factor rows (warp per row, fused
row sort), CSR packing, optional factor compression with validation, and the
explicit transpose.  Apply is the fused G -> G^T product.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib
from .linear import LinearOperator
from .sparse import BsrMatrix, bsr_transposed, scalarize

_PIVOT_FLOOR = {torch.float32: 1.0e-6, torch.float64: 1.0e-12}


def fsai_rows(scalar: BsrMatrix, width: int, step: int, kap: float, pivot_floor: float):
    """Adaptive factor rows: returns (ell_cols, ell_vals, row_counts, scale, status[3])."""
    n = scalar.nrow
    dev = scalar.device
    dt = scalar.scalar_type
    cols = torch.empty(n * width, dtype=torch.int32, device=dev)
    vals = torch.empty(n * width, dtype=dt, device=dev)
    counts = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    scale = torch.empty(max(n, 1), dtype=dt, device=dev)
    status = (ctypes.c_int32 * 3)()
    rc = _lib.load().gbpc_fsai_setup(
        n, _lib.ptr(scalar.offsets), _lib.ptr(scalar.columns), _lib.ptr(scalar.values),
        _lib.dtype_code(dt), width, step, float(kap), float(pivot_floor), _lib.ptr(cols),
        _lib.ptr(vals), _lib.ptr(counts), _lib.ptr(scale), status, _lib.stream(dev))
    return cols, vals, counts, scale, list(status), rc


def pack_rows(n, width, cols, vals, counts) -> BsrMatrix:
    """Sorted ELL rows -> canonical CSR (fsai_pack.py:58-71)."""
    dev = vals.device
    off = torch.empty(n + 1, dtype=torch.int32, device=dev)
    nnz = ctypes.c_int64()
    code = _lib.dtype_code(vals.dtype)
    _lib.call("gbpc_fsai_pack", n, width, _lib.ptr(cols), _lib.ptr(vals), _lib.ptr(counts), code,
              _lib.ptr(off), None, None, ctypes.byref(nnz), _lib.stream(dev))
    col = torch.empty(nnz.value, dtype=torch.int32, device=dev)
    val = torch.empty(nnz.value, dtype=vals.dtype, device=dev)
    _lib.call("gbpc_fsai_pack", n, width, _lib.ptr(cols), _lib.ptr(vals), _lib.ptr(counts), code,
              _lib.ptr(off), _lib.ptr(col), _lib.ptr(val), ctypes.byref(nnz), _lib.stream(dev))
    return BsrMatrix(n, n, (1, 1), off, col, val)


def convert_factor(g: BsrMatrix, dtype: torch.dtype) -> BsrMatrix:
    """Narrow the factor storage and validate it (fsai.py:181-196, :343-355)."""
    out = torch.empty(g.nnz, dtype=dtype, device=g.device)
    bad = ctypes.c_int32()
    _lib.call("gbpc_convert_factor", g.nrow, _lib.ptr(g.offsets), _lib.ptr(g.columns),
              _lib.ptr(g.values), _lib.dtype_code(g.scalar_type), _lib.ptr(out),
              _lib.dtype_code(dtype), ctypes.byref(bad), _lib.stream(g.device), what="FSAI")
    return BsrMatrix(g.nrow, g.ncol, (1, 1), g.offsets, g.columns, out)


class FSAI(LinearOperator):
    """Approximate inverse ``G.T @ G`` of an SPD BSR matrix.

    Same constructor as warp_preconditioners.FSAI (fsai.py:241-251):
    ``max_row_size`` includes the diagonal; each search selects up to
    ``max_step_size`` distinct largest-residual entries from the lower
    triangular frontier; ``kap_tolerance`` tests the relative energy
    improvement after each batch (zero disables it); square blocks are
    scalarised keeping stored zeros.  float32 and float64 matrices are
    supported.  ``factor_dtype`` may be the matrix type, float32 for a float64
    matrix (products still accumulate in float64), or bfloat16 (an addition of
    this build for the mixed-precision path).  ``apply_lanes`` is validated for
    compatibility; the apply kernel's layout is chosen by the library.
    Setup synchronises; apply is stream-ordered and graph-capturable.  With
    ``reuse_pattern=True``, ``update(A)`` refits the original supports for new
    values on the same topology (fsai_reuse.py).

    ``apply_dtype=torch.float32`` (an addition of this build; float64
    matrices only) applies the factor with float32 arithmetic behind the
    float64 vector interface: G stored in float32 (or bfloat16 with
    ``factor_dtype=torch.bfloat16``), the input narrowed, products summed in
    float32, the result widened.  Inside ``linear.cg`` / ``Solver`` the
    conversions are fused into the loop's own vector kernels, so the
    preconditioner streams half (bfloat16: three eighths) of the float64
    factor's bytes and issues no float64 arithmetic, while the Krylov
    recurrences, dot products and the system operator stay float64.
    """

    def __init__(self, A, max_row_size=8, kap_tolerance=1.0e-3, pivot_floor=None, apply_lanes=1,
                 factor_dtype=None, reuse_pattern=False, max_step_size=1, apply_dtype=None):
        if (not isinstance(A, BsrMatrix) or A.shape[0] != A.shape[1]
                or A.block_shape[0] != A.block_shape[1]):
            raise ValueError("FSAI requires a square BSR matrix with square blocks")
        if A.scalar_type not in (torch.float32, torch.float64):
            raise TypeError("FSAI supports float32 and float64")
        if isinstance(max_row_size, bool) or not isinstance(max_row_size, int) \
                or not 1 <= max_row_size <= 64:
            raise ValueError("max_row_size must be an integer in [1, 64]")
        if isinstance(max_step_size, bool) or not isinstance(max_step_size, int) \
                or not 1 <= max_step_size <= 64:
            raise ValueError("max_step_size must be an integer in [1, 64]")
        if not 0 <= kap_tolerance < 1:
            raise ValueError("kap_tolerance must be in [0, 1)")
        if pivot_floor is None:
            pivot_floor = _PIVOT_FLOOR[A.scalar_type]
        if not 0 < pivot_floor < 1:
            raise ValueError("pivot_floor must be in (0, 1)")
        if not isinstance(apply_lanes, int) or apply_lanes not in (1, 2, 4, 8, 16, 32):
            raise ValueError("apply_lanes must be one of 1, 2, 4, 8, 16, 32")
        if apply_dtype not in (None, A.scalar_type, torch.float32):
            raise ValueError("apply_dtype must be the matrix scalar type or torch.float32")
        low = apply_dtype == torch.float32 and A.scalar_type == torch.float64
        if factor_dtype is None:
            factor_dtype = torch.float32 if low else A.scalar_type
        if low and factor_dtype not in (torch.float32, torch.bfloat16):
            raise ValueError("apply_dtype=torch.float32 needs float32 or bfloat16 factor storage")
        if factor_dtype != A.scalar_type and not (
            A.scalar_type == torch.float64 and factor_dtype in (torch.float32, torch.bfloat16)
        ):
            raise ValueError(
                "factor_dtype must be the matrix scalar type, or torch.float32 for a float64 matrix"
            )
        self.max_row_size = max_row_size
        self.max_step_size = max_step_size
        self.factor_dtype = factor_dtype
        self.apply_lanes = apply_lanes
        self.source = A
        scalar = scalarize(A)
        n = scalar.nrow
        dt = scalar.scalar_type
        cols, vals, counts, scale, status, rc = fsai_rows(scalar, max_row_size, max_step_size,
                                                          kap_tolerance, pivot_floor)
        if rc == _lib.ERR_DIAGONAL or status[0]:
            raise ValueError(f"FSAI requires finite positive diagonals ({status[0]} invalid rows)")
        if rc == _lib.ERR_FACTOR or status[2]:
            raise ValueError("FSAI factor lost finite entries or a positive diagonal")
        _lib.check(rc, "FSAI")
        self.truncated_rows = int(status[1])
        self.scale = scale[:n]
        self.G = pack_rows(n, max_row_size, cols, vals, counts)
        if factor_dtype != dt:
            self.G = convert_factor(self.G, factor_dtype)
        self.GT = bsr_transposed(self.G)
        self._op = _lib.new_op(
            "gbpc_op_fsai", n, 1, _lib.ptr(self.G.offsets), _lib.ptr(self.G.columns),
            _lib.ptr(self.G.values), _lib.ptr(self.GT.offsets), _lib.ptr(self.GT.columns),
            _lib.ptr(self.GT.values), _lib.dtype_code(factor_dtype),
            _lib.GBPC_F32_APPLY if low else _lib.dtype_code(dt), _lib.stream(A.device))
        self.apply_dtype = torch.float32 if low else dt
        super().__init__(A.shape, dt, A.device, self._apply)
        self._refit = _RefitPlan(self, A, max_row_size, pivot_floor) if reuse_pattern else None

    def update(self, A=None):
        """Refit on the original factor supports (fsai.py:346-362).

        Requires ``reuse_pattern=True`` and the topology the factor was built
        from.  This is not a new adaptive pattern search; rebuild when
        convergence worsens.  A failed validation leaves the previous factor
        intact.  G and GT keep their storage, so captured applies see the new
        values.  Synchronises.
        """
        if self._refit is None:
            raise ValueError("Construct FSAI with reuse_pattern=True before updating")
        A = self.source if A is None else A
        if not isinstance(A, BsrMatrix):
            raise ValueError("update requires a BsrMatrix")
        self._refit.update(self, A)
        self.source = A
        return self

    def quality(self, A=None, probes=4, seed=17):
        """Rademacher estimate of ``||G A G^T - I||_F / sqrt(n)`` with fixed
        random probes (fsai_reuse.py:248-279): a diagnostic, not a bound on
        conditioning or iterations.  Probe p is the reference's seeded
        stream (``rand_init(seed + p, i)``, fsai_reuse.py:143-147) drawn on
        the device; the products, the subtraction and the float64 dot run in
        libgbpc.  Allocates and synchronises once; not capturable."""
        if isinstance(probes, bool) or not isinstance(probes, int) or probes < 1:
            raise ValueError("probes must be a positive integer")
        A = self.source if A is None else A
        if (not isinstance(A, BsrMatrix)
                or (A.shape, A.dtype, A.device) != (self.shape, self.dtype, self.device)):
            raise ValueError("quality requires matching shape, dtype and device")
        n = A.shape[0]
        if n == 0:
            return 0.0
        from .linear import aslinearoperator

        dt = A.scalar_type
        code = _lib.dtype_code(dt)
        g_op, gt_op = _product_op(self.G, dt), _product_op(self.GT, dt)
        a_op = aslinearoperator(A)
        x, y, z, w = (torch.empty(n, dtype=dt, device=A.device) for _ in range(4))
        work = torch.empty(_lib.load().gbpc_vec_dot_work_size(), dtype=torch.float64,
                           device=A.device)
        dots = torch.empty(probes, dtype=torch.float64, device=A.device)
        st = _lib.stream(A.device)
        for p in range(probes):
            _lib.call("gbpc_rademacher", n, seed + p, code, _lib.ptr(x), st)
            gt_op.apply(x, None, y, 1.0, 0.0, A.device)
            a_op.matvec(y, None, z, 1.0, 0.0)
            g_op.apply(z, None, w, 1.0, 0.0, A.device)
            _lib.call("gbpc_vec_axpby", n, code, 1.0, _lib.ptr(w), -1.0, _lib.ptr(x),
                      _lib.ptr(w), st)
            _lib.call("gbpc_vec_dot", n, code, _lib.ptr(w), _lib.ptr(w), _lib.ptr(work),
                      ctypes.c_void_p(dots.data_ptr() + 8 * p), st)
        total = 0.0
        for d in dots.tolist():  # the reference adds the probes' dots in order on the host
            total += d
        return (total / (probes * max(n, 1))) ** 0.5

    def _apply(self, x, y, z, alpha, beta):
        self._op.apply(x.reshape(-1), y.reshape(-1) if y is not None else None, z.view(-1),
                       alpha, beta, self.device)


def _product_op(M: BsrMatrix, vector_dtype) -> _lib.OpHandle:
    """Plain product with M (scalar CSR) on vectors of `vector_dtype`."""
    return _lib.new_op("gbpc_op_sparse", M.nrow, M.ncol, 1, _lib.ptr(M.offsets),
                       _lib.ptr(M.columns), _lib.ptr(M.values), _lib.dtype_code(M.scalar_type),
                       _lib.dtype_code(vector_dtype), _lib.stream(M.device))


class _RefitPlan:
    """Fixed-support refit state (fsai_reuse.py:157-245, ``RefitPlan``): the
    source topology to compare against, the position of every G entry in
    G^T, and a candidate buffer that replaces G's values only when every row
    of the refit is valid."""

    def __init__(self, owner: FSAI, A: BsrMatrix, width: int, floor: float):
        self.signature = (A.shape, A.block_shape, A.scalar_type, A.device)
        self.offsets = A.offsets.clone()
        self.columns = A.columns.clone()
        self.width, self.floor = width, float(floor)
        G, GT = owner.G, owner.GT
        self.transpose = torch.empty(max(G.nnz, 1), dtype=torch.int32, device=A.device)
        if G.nnz:
            _lib.call("gbpc_transpose_map", G.nrow, _lib.ptr(G.offsets), _lib.ptr(G.columns),
                      _lib.ptr(GT.offsets), _lib.ptr(GT.columns), _lib.ptr(self.transpose),
                      _lib.stream(A.device))
        self.candidate = torch.empty_like(G.values)

    def update(self, owner: FSAI, A: BsrMatrix) -> None:
        if (A.shape, A.block_shape, A.scalar_type, A.device) != self.signature:
            raise ValueError("FSAI update requires the original shape, dtype, device and topology")
        if A.offsets.shape != self.offsets.shape or A.columns.shape != self.columns.shape:
            raise ValueError("FSAI update requires identical topology storage")
        if not (torch.equal(A.offsets, self.offsets) and torch.equal(A.columns, self.columns)):
            raise ValueError("FSAI update requires identical sparsity; rebuild to change it")
        if A.values.numel() < self.columns.numel() * A.block_size:
            raise ValueError("Insufficient source values")
        G, GT = owner.G, owner.GT
        if G.nrow == 0:
            return
        scalar = scalarize(A)
        st = _lib.stream(A.device)
        status = (ctypes.c_int32 * 2)()
        _lib.call("gbpc_fsai_refit", G.nrow, _lib.ptr(scalar.offsets), _lib.ptr(scalar.columns),
                  _lib.ptr(scalar.values.reshape(-1)), _lib.dtype_code(scalar.scalar_type),
                  _lib.ptr(G.offsets), _lib.ptr(G.columns), self.width, self.floor,
                  _lib.ptr(self.candidate), _lib.dtype_code(G.scalar_type), status, st)
        if status[0] or status[1]:
            raise ValueError("FSAI refit requires finite positive diagonals and SPD local supports")
        G.values.copy_(self.candidate)
        _lib.call("gbpc_scatter_values", G.nnz, _lib.ptr(G.values), _lib.ptr(self.transpose),
                  _lib.ptr(GT.values), _lib.dtype_code(G.scalar_type), st)
        _lib.call("gbpc_op_fsai_refill", owner._op.handle, _lib.ptr(G.offsets),
                  _lib.ptr(G.columns), _lib.ptr(G.values), _lib.ptr(GT.offsets),
                  _lib.ptr(GT.columns), _lib.ptr(GT.values), _lib.dtype_code(G.scalar_type), st)
