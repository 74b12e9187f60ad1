"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle restates the reference algorithms of alecjacobson/warp-preconditioners
in sequential C++ (``gbpc_oracle.cpp``).  Only ``tests/``, the smoke check and
the CPU-baseline leg of ``bench.py`` import this module, always as the checker,
never as the thing measured or shipped.

Parity pin: the reference ships no golden vectors; its tests generate known
answers.  ``tests/golden/make_golden.py`` restates those known-answer
computations with dense NumPy (independent of this oracle) and the
``tests/test_oracle_*.py`` files check the oracle against the fixtures.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"

_i32p = ctypes.POINTER(ctypes.c_int32)
_f64p = ctypes.POINTER(ctypes.c_double)
_f32p = ctypes.POINTER(ctypes.c_float)


def build(force: bool = False) -> Path:
    """Compile the oracle with its Makefile (g++, -ffp-contract=off)."""
    src = HERE / "gbpc_oracle.cpp"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(str(LIB_PATH))
        _lib.or_fsai_pack_f64.restype = ctypes.c_int64
        _lib.or_fsai_pack_f32.restype = ctypes.c_int64
    return _lib


def set_threads(n: int) -> None:
    lib().or_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().or_num_threads())


def _p(a: np.ndarray):
    if a is None:
        return None
    assert a.flags.c_contiguous, "oracle arrays must be contiguous"
    if a.dtype == np.int32:
        return a.ctypes.data_as(_i32p)
    if a.dtype == np.float64:
        return a.ctypes.data_as(_f64p)
    if a.dtype == np.float32:
        return a.ctypes.data_as(_f32p)
    raise TypeError(a.dtype)


def _sfx(dtype) -> str:
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


def _scalar(dtype, v):
    return ctypes.c_double(v) if np.dtype(dtype) == np.float64 else ctypes.c_float(v)


class CSR:
    """Canonical scalar CSR on the host (sorted, unique columns)."""

    def __init__(self, offsets, columns, values, ncol=None):
        self.offsets = np.ascontiguousarray(offsets, dtype=np.int32)
        self.columns = np.ascontiguousarray(columns, dtype=np.int32)
        self.values = np.ascontiguousarray(values)
        self.nrow = len(self.offsets) - 1
        self.ncol = self.nrow if ncol is None else ncol

    @classmethod
    def from_scipy(cls, a, dtype=np.float64):
        import scipy.sparse as ss

        a = ss.csr_matrix(a)
        a.sum_duplicates()
        a.sort_indices()
        return cls(a.indptr, a.indices, a.data.astype(dtype), a.shape[1])

    def to_scipy(self):
        import scipy.sparse as ss

        return ss.csr_matrix(
            (self.values, self.columns, self.offsets), shape=(self.nrow, self.ncol)
        )


def fsai_setup(a: CSR, width=8, step=1, tol=1e-3, pivot_floor=None):
    """fsai.py:44-176 — returns (ell_cols, ell_vals, scale, status[3])."""
    dtype = a.values.dtype
    if pivot_floor is None:
        pivot_floor = 1e-12 if dtype == np.float64 else 1e-6
    n = a.nrow
    cols = np.empty(n * width, np.int32)
    vals = np.empty(n * width, dtype)
    scale = np.empty(n, dtype)
    status = np.zeros(3, np.int32)
    getattr(lib(), "or_fsai_setup_" + _sfx(dtype))(
        n, _p(a.offsets), _p(a.columns), _p(a.values), width, step,
        _scalar(dtype, tol), _scalar(dtype, pivot_floor), _p(cols), _p(vals), _p(scale), _p(status),
    )
    return cols, vals, scale, status


def fsai_rows(a: CSR, rows, width=8, step=1, tol=1e-3, pivot_floor=None):
    """The float64 FSAI rows `rows` only (fsai.py:60-176 builds every row
    independently): returns (columns, values) per listed row, each sorted by
    column like the packed factor (fsai_pack.py:15-71), and status[3]."""
    a = CSR(a.offsets, a.columns, np.ascontiguousarray(a.values, np.float64), a.ncol)
    if pivot_floor is None:
        pivot_floor = 1e-12
    rows = np.ascontiguousarray(rows, np.int32)
    cols = np.empty(max(len(rows), 1) * width, np.int32)
    vals = np.empty(max(len(rows), 1) * width, np.float64)
    status = np.zeros(3, np.int32)
    lib().or_fsai_setup_rows_f64(a.nrow, _p(a.offsets), _p(a.columns), _p(a.values), width, step,
                                 ctypes.c_double(tol), ctypes.c_double(pivot_floor), len(rows),
                                 _p(rows), _p(cols), _p(vals), _p(status))
    out = []
    for k in range(len(rows)):
        c = cols[k * width:(k + 1) * width]
        v = vals[k * width:(k + 1) * width]
        keep = c >= 0
        order = np.argsort(c[keep], kind="stable")
        out.append((c[keep][order], v[keep][order]))
    return out, status


def fsai_setup_flops(a: CSR, width=8, step=1, tol=1e-3, pivot_floor=None):
    """Floating-point operations of the float64 FSAI setup (fsai.py:44-176),
    counted while the oracle runs it: each separately rounded multiply,
    add/subtract, divide and square root is one (the reference evaluates
    without contraction).  Returns (flops, ell_cols, ell_vals)."""
    a = CSR(a.offsets, a.columns, np.ascontiguousarray(a.values, np.float64), a.ncol)
    if pivot_floor is None:
        pivot_floor = 1e-12
    n = a.nrow
    cols = np.empty(n * width, np.int32)
    vals = np.empty(n * width, np.float64)
    scale = np.empty(n, np.float64)
    status = np.zeros(3, np.int32)
    fn = lib().or_fsai_setup_flops_f64
    fn.restype = ctypes.c_int64
    flops = fn(n, _p(a.offsets), _p(a.columns), _p(a.values), width, step,
               ctypes.c_double(tol), ctypes.c_double(pivot_floor), _p(cols), _p(vals), _p(scale),
               _p(status))
    return int(flops), cols, vals


def fsai_pack(n, width, ell_cols, ell_vals):
    """fsai_pack.py:15-71 — sorts the ELL rows in place, returns CSR G."""
    ell_cols = np.ascontiguousarray(ell_cols, np.int32).copy()
    ell_vals = np.ascontiguousarray(ell_vals).copy()
    off = np.empty(n + 1, np.int32)
    fn = getattr(lib(), "or_fsai_pack_" + _sfx(ell_vals.dtype))
    nnz = fn(n, width, _p(ell_cols), _p(ell_vals), _p(off), None, None)
    col = np.empty(nnz, np.int32)
    val = np.empty(nnz, ell_vals.dtype)
    fn(n, width, _p(ell_cols), _p(ell_vals), _p(off), _p(col), _p(val))
    return CSR(off, col, val)


def transpose(a: CSR) -> CSR:
    t_off = np.empty(a.ncol + 1, np.int32)
    t_col = np.empty(len(a.columns), np.int32)
    t_val = np.empty(len(a.values), a.values.dtype)
    getattr(lib(), "or_csr_transpose_" + _sfx(a.values.dtype))(
        a.nrow, a.ncol, _p(a.offsets), _p(a.columns), _p(a.values), _p(t_off), _p(t_col), _p(t_val)
    )
    return CSR(t_off, t_col, t_val, a.nrow)


def scalarize(nrow_blocks, b, offsets, columns, values) -> CSR:
    """fsai_pack.py:74-107 — b x b BSR (values shaped [nnzb, b, b]) to CSR."""
    values = np.ascontiguousarray(values)
    nnzb = int(offsets[-1])
    out_off = np.empty(nrow_blocks * b + 1, np.int32)
    out_col = np.empty(nnzb * b * b, np.int32)
    out_val = np.empty(nnzb * b * b, values.dtype)
    getattr(lib(), "or_scalarize_" + _sfx(values.dtype))(
        nrow_blocks, b, _p(np.ascontiguousarray(offsets, np.int32)),
        _p(np.ascontiguousarray(columns, np.int32)), _p(values.reshape(-1)),
        _p(out_off), _p(out_col), _p(out_val),
    )
    return CSR(out_off, out_col, out_val, nrow_blocks * b)


def fsai(a: CSR, width=8, step=1, tol=1e-3, pivot_floor=None, factor_dtype=None):
    """Full FSAI setup (fsai.py:241-358): returns (G, GT, truncated_rows)."""
    cols, vals, _, status = fsai_setup(a, width, step, tol, pivot_floor)
    if status[0]:
        raise ValueError(f"FSAI requires finite positive diagonals ({status[0]} invalid rows)")
    if status[2]:
        raise ValueError("FSAI factor lost finite entries or a positive diagonal")
    g = fsai_pack(a.nrow, width, cols, vals)
    if factor_dtype is not None and np.dtype(factor_dtype) != g.values.dtype:
        g = CSR(g.offsets, g.columns, g.values.astype(factor_dtype))
    return g, transpose(g), int(status[1])


def fsai_refit(a: CSR, g: CSR, pivot_floor=None, factor_dtype=None):
    """fsai_reuse.py:189-245 (RefitPlan.update: `diagonal` then `refit`) on the
    fixed supports of G.  Returns (values in G's layout, invalid diagonals,
    invalid rows); the caller publishes the values only when both are 0."""
    dtype = a.values.dtype
    if pivot_floor is None:
        pivot_floor = 1e-12 if dtype == np.float64 else 1e-6
    out_dtype = np.dtype(factor_dtype) if factor_dtype is not None else dtype
    n = a.nrow
    scale = np.empty(max(n, 1), dtype)
    status = np.zeros(1, np.int32)
    getattr(lib(), "or_fsai_diagonal_" + _sfx(dtype))(
        n, _p(a.offsets), _p(a.columns), _p(a.values), _p(scale), _p(status))
    out = np.empty(max(len(g.columns), 1), out_dtype)
    fn = getattr(lib(), f"or_fsai_refit_{_sfx(dtype)}_{_sfx(out_dtype)}")
    fn.restype = ctypes.c_int32
    bad = fn(n, _p(a.offsets), _p(a.columns), _p(a.values), _p(scale),
             _p(np.ascontiguousarray(g.offsets, np.int32)),
             _p(np.ascontiguousarray(g.columns, np.int32)), _scalar(dtype, pivot_floor), _p(out))
    return out[:len(g.columns)], int(status[0]), int(bad)


def spgemm(a: CSR, b: CSR, col_scale=None, add_diag=None) -> CSR:
    """SciPy's order for A @ diags(d) @ B + diags(e) (the reference's host
    assembly of Q: inner index decreasing), separately rounded; sorted CSR."""
    fn = lib().or_spgemm
    fn.restype = ctypes.c_int64
    d = None if col_scale is None else np.ascontiguousarray(col_scale, np.float64)
    e = None if add_diag is None else np.ascontiguousarray(add_diag, np.float64)
    off = np.empty(a.nrow + 1, np.int32)
    args = [a.nrow, b.ncol, _p(a.offsets), _p(a.columns), _p(a.values), _p(d), _p(b.offsets),
            _p(b.columns), _p(b.values), _p(e), _p(off)]
    nnz = fn(*args, None, None)
    col = np.empty(max(nnz, 1), np.int32)
    val = np.empty(max(nnz, 1))
    fn(*args, _p(col), _p(val))
    return CSR(off, col[:nnz], val[:nnz], b.ncol)


def csr_spmv(a: CSR, x, y, alpha, beta, accum_dtype=None):
    accum_dtype = np.dtype(accum_dtype or a.values.dtype)
    x = np.ascontiguousarray(x, accum_dtype)
    y = np.ascontiguousarray(y, accum_dtype)
    z = np.empty(a.nrow, accum_dtype)
    if a.values.dtype == np.float32 and accum_dtype == np.float64:
        fn = lib().or_csr_spmv_f32s_f64a
    else:
        fn = getattr(lib(), "or_csr_spmv_" + _sfx(accum_dtype))
    fn(a.nrow, _p(a.offsets), _p(a.columns), _p(a.values), _p(x), _p(y), _p(z),
       _scalar(accum_dtype, alpha), _scalar(accum_dtype, beta))
    return z


def fsai_apply(g: CSR, gt: CSR, x, y, alpha, beta, accum_dtype=np.float64):
    tmp = csr_spmv(g, x, np.zeros(g.nrow, accum_dtype), 1.0, 0.0, accum_dtype)
    return csr_spmv(gt, tmp, y, alpha, beta, accum_dtype)


def _pcg_hash(v):
    """The PCG hash (Jarzynski and Olano, JCGT 9(3), 2020) on uint32 arrays."""
    v = np.asarray(v, np.uint32)
    with np.errstate(over="ignore"):
        state = v * np.uint32(747796405) + np.uint32(2891336453)
        word = ((state >> ((state >> np.uint32(28)) + np.uint32(4))) ^ state) * np.uint32(277803737)
    return (word >> np.uint32(22)) ^ word


def rademacher(n, seed, dtype=np.float64):
    """Probe of FSAI.quality, warp_preconditioners/fsai_reuse.py:143-147:
    out[i] = 2 randi(rand_init(seed, i), 0, 2) - 1, with Warp's
    rand_init(seed, i) = pcg(seed + pcg(i)) and randi advancing the state by
    one hash and returning lo + state % (hi - lo)."""
    i = np.arange(n, dtype=np.uint32)
    with np.errstate(over="ignore"):
        state = _pcg_hash(np.uint32(seed & 0xFFFFFFFF) + _pcg_hash(i))
    draw = _pcg_hash(state)
    return (2 * (draw % np.uint32(2)).astype(np.int64) - 1).astype(dtype)


def fsai_quality(a: CSR, g: CSR, gt: CSR, probes=4, seed=17):
    """||G A G^T - I||_F / sqrt(n) estimated with the reference's probes
    (warp_preconditioners/fsai_reuse.py:248-279): per probe x,
    w = G (A (G^T x)) - x and total += w.w; result sqrt(total / (probes n))."""
    n = a.nrow
    if n == 0:
        return 0.0
    dt = a.values.dtype
    zero = np.zeros(n, dt)
    total = 0.0
    for p in range(probes):
        x = rademacher(n, seed + p, dt)
        y = csr_spmv(gt, x, zero, 1.0, 0.0, dt)
        z = csr_spmv(a, y, zero, 1.0, 0.0, dt)
        w = csr_spmv(g, z, zero, 1.0, 0.0, dt) - x
        total += float(np.dot(w.astype(np.float64), w.astype(np.float64)))
    return (total / (probes * n)) ** 0.5


def bsr_spmv(nrow, b, offsets, columns, values, x, y, alpha, beta):
    values = np.ascontiguousarray(values)
    x = np.ascontiguousarray(x, np.float64).reshape(-1)
    y = np.ascontiguousarray(y, np.float64).reshape(-1)
    z = np.empty(nrow * b, np.float64)
    fn = lib().or_bsr_spmv_f64 if values.dtype == np.float64 else lib().or_bsr_spmv_f32s_f64a
    fn(nrow, b, _p(np.ascontiguousarray(offsets, np.int32)),
       _p(np.ascontiguousarray(columns, np.int32)), _p(values.reshape(-1)),
       _p(x), _p(y), _p(z), ctypes.c_double(alpha), ctypes.c_double(beta))
    return z


def sqlap_apply(L: CSR, mass, free, mass_weight, x, y, alpha, beta, boundary=False):
    """squared_laplacian.py:37-101 forward + backward."""
    dtype = L.values.dtype
    mass = np.ascontiguousarray(mass, dtype)
    free = np.ascontiguousarray(free, np.int32)
    index = np.full(L.nrow, -1, np.int32)
    index[free] = np.arange(len(free), dtype=np.int32)
    inv = (1 / mass).astype(dtype)
    x = np.ascontiguousarray(x, dtype)
    y = np.ascontiguousarray(y, dtype)
    z = np.empty(len(free), dtype)
    tmp = np.empty(L.nrow, dtype)
    getattr(lib(), "or_sqlap_apply_" + _sfx(dtype))(
        L.nrow, _p(L.offsets), _p(L.columns), _p(L.values), _p(inv), _p(mass), _p(free),
        len(free), _p(index), _scalar(dtype, mass_weight), _p(x), _p(y), _p(z),
        _scalar(dtype, alpha), _scalar(dtype, beta), int(boundary), _p(tmp),
    )
    return z


def block_diag_inverse(nrow, b, offsets, columns, values, tol=None):
    values = np.ascontiguousarray(values)
    if tol is None:
        tol = 1e-12 if values.dtype == np.float64 else 1e-6
    inv = np.empty((nrow, b, b), values.dtype)
    bad = getattr(lib(), "or_block_diag_inverse_" + _sfx(values.dtype))(
        nrow, b, _p(np.ascontiguousarray(offsets, np.int32)),
        _p(np.ascontiguousarray(columns, np.int32)), _p(values.reshape(-1)),
        _scalar(values.dtype, tol), _p(inv.reshape(-1)),
    )
    return inv, int(bad)


def bilu0_setup(nrow, b, offsets, columns, values, factor_sweeps=12, relaxation=1.0, tol=None):
    values = np.ascontiguousarray(values)
    if tol is None:
        tol = 1e-12 if values.dtype == np.float64 else 1e-6
    nnzb = int(offsets[-1])
    factors = np.empty((nnzb, b, b), values.dtype)
    inv = np.empty((nrow, b, b), values.dtype)
    bad = getattr(lib(), "or_bilu0_setup_" + _sfx(values.dtype))(
        nrow, b, _p(np.ascontiguousarray(offsets, np.int32)),
        _p(np.ascontiguousarray(columns, np.int32)), _p(values.reshape(-1)), factor_sweeps,
        _scalar(values.dtype, relaxation), _scalar(values.dtype, tol),
        _p(factors.reshape(-1)), _p(inv.reshape(-1)),
    )
    return factors, inv, int(bad)


def bilu0_apply(nrow, b, offsets, columns, factors, inverse, solve_sweeps, x, y, alpha, beta):
    dtype = factors.dtype
    x = np.ascontiguousarray(x, dtype).reshape(-1)
    y = np.ascontiguousarray(y, dtype).reshape(-1)
    z = np.empty(nrow * b, dtype)
    getattr(lib(), "or_bilu0_apply_" + _sfx(dtype))(
        nrow, b, _p(np.ascontiguousarray(offsets, np.int32)),
        _p(np.ascontiguousarray(columns, np.int32)), _p(np.ascontiguousarray(factors).reshape(-1)),
        _p(np.ascontiguousarray(inverse).reshape(-1)), solve_sweeps, _p(x), _p(y), _p(z),
        _scalar(dtype, alpha), _scalar(dtype, beta),
    )
    return z


def block_jacobi_apply(inverse, x, y, alpha, beta):
    nrow, b, _ = inverse.shape
    x = np.ascontiguousarray(x, np.float64).reshape(-1)
    y = np.ascontiguousarray(y, np.float64).reshape(-1)
    z = np.empty(nrow * b)
    lib().or_block_jacobi_apply_f64(nrow, b, _p(np.ascontiguousarray(inverse).reshape(-1)),
                                    _p(x), _p(y), _p(z), ctypes.c_double(alpha),
                                    ctypes.c_double(beta))
    return z


def block_fsai_setup(nrow, b, max_blocks, offsets, columns, values, refit_cols=None):
    """block_fsai_candidate.py:45-178 — returns (ell_cols, ell_vals, scale, bad)."""
    width = b * max_blocks
    n = nrow * b
    cols = np.empty(n * width, np.int32) if refit_cols is None else refit_cols.copy()
    vals = np.empty(n * width, np.float64)
    scale = np.empty(n, np.float64)
    bad = lib().or_block_fsai_setup_f64(
        nrow, b, max_blocks, _p(np.ascontiguousarray(offsets, np.int32)),
        _p(np.ascontiguousarray(columns, np.int32)),
        _p(np.ascontiguousarray(values, np.float64).reshape(-1)),
        _p(cols), _p(vals), _p(scale), int(refit_cols is not None),
    )
    return cols, vals, scale, int(bad)


# --- Krylov -----------------------------------------------------------------


class _Op(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int), ("n", ctypes.c_int), ("nrow", ctypes.c_int), ("b", ctypes.c_int),
        ("off", ctypes.c_void_p), ("col", ctypes.c_void_p), ("val", ctypes.c_void_p),
        ("val_f32", ctypes.c_int),
        ("off2", ctypes.c_void_p), ("col2", ctypes.c_void_p), ("val2", ctypes.c_void_p),
        ("mass", ctypes.c_void_p), ("inv_mass", ctypes.c_void_p), ("mass_weight", ctypes.c_double),
        ("diag", ctypes.c_void_p), ("factors", ctypes.c_void_p), ("sweeps", ctypes.c_int),
    ]


class Operator:
    """Host operator description for the oracle's PCG / PCR loops."""

    def __init__(self, kind, n, **arrays):
        self._keep = []
        s = _Op()
        s.kind, s.n = kind, n
        s.nrow = arrays.pop("nrow", n)
        s.b = arrays.pop("b", 1)
        s.mass_weight = arrays.pop("mass_weight", 0.0)
        s.sweeps = arrays.pop("sweeps", 0)
        for name, arr in arrays.items():
            if arr is None:
                continue
            arr = np.ascontiguousarray(arr)
            self._keep.append(arr)
            if name in ("val", "val2") and arr.dtype == np.float32:
                s.val_f32 = 1
            setattr(s, name, arr.ctypes.data)
        self.s = s

    @classmethod
    def csr(cls, a: CSR):
        return cls(1, a.nrow, off=a.offsets, col=a.columns, val=a.values)

    @classmethod
    def bsr(cls, nrow, b, offsets, columns, values):
        return cls(2, nrow * b, nrow=nrow, b=b, off=np.asarray(offsets, np.int32),
                   col=np.asarray(columns, np.int32), val=np.asarray(values).reshape(-1))

    @classmethod
    def sqlap(cls, L: CSR, mass, mass_weight):
        mass = np.asarray(mass, np.float64)
        return cls(3, L.nrow, off=L.offsets, col=L.columns, val=L.values, mass=mass,
                   inv_mass=1 / mass, mass_weight=mass_weight)

    @classmethod
    def fsai(cls, g: CSR, gt: CSR):
        return cls(4, g.nrow, off=g.offsets, col=g.columns, val=g.values, off2=gt.offsets,
                   col2=gt.columns, val2=gt.values)

    @classmethod
    def diagonal(cls, d_inv):
        return cls(5, len(d_inv), diag=np.asarray(d_inv, np.float64))

    @classmethod
    def block_jacobi(cls, inverse):
        nrow, b, _ = inverse.shape
        return cls(6, nrow * b, nrow=nrow, b=b, diag=inverse.reshape(-1))

    @classmethod
    def bilu0(cls, nrow, b, offsets, columns, factors, inverse, solve_sweeps):
        return cls(7, nrow * b, nrow=nrow, b=b, off=np.asarray(offsets, np.int32),
                   col=np.asarray(columns, np.int32), factors=factors.reshape(-1),
                   diag=inverse.reshape(-1), sweeps=solve_sweeps)

    def apply(self, x, y, alpha, beta):
        x = np.ascontiguousarray(x, np.float64).reshape(-1)
        y = np.ascontiguousarray(y, np.float64).reshape(-1)
        z = np.empty(self.s.n)
        lib().or_operator_apply(ctypes.byref(self.s), _p(x), _p(y), _p(z),
                                ctypes.c_double(alpha), ctypes.c_double(beta))
        return z


def krylov(method, A: Operator, b, x0=None, M: Operator | None = None, tol=1e-8, atol=0.0,
           maxiter=10000):
    """Textbook PCG (method 'cg') or PCR ('cr'); returns (x, iterations, rr, atol_sq)."""
    b = np.ascontiguousarray(b, np.float64).reshape(-1)
    x = np.zeros_like(b) if x0 is None else np.ascontiguousarray(x0, np.float64).reshape(-1).copy()
    rr = ctypes.c_double()
    atol_sq = ctypes.c_double()
    fn = lib().or_krylov_f64
    fn.restype = ctypes.c_int
    it = fn(0 if method == "cg" else 1, ctypes.byref(A.s),
            ctypes.byref(M.s) if M is not None else None, _p(b), _p(x),
            ctypes.c_double(tol), ctypes.c_double(atol), int(maxiter),
            ctypes.byref(rr), ctypes.byref(atol_sq))
    return x, int(it), rr.value, atol_sq.value


def gmres(A: Operator, b, x0=None, M: Operator | None = None, tol=1e-5, atol=0.0, restart=31,
          maxiter=0):
    """Textbook restarted right-preconditioned GMRES(restart) in numpy (small
    cases): Arnoldi on A M with classical Gram-Schmidt applied twice, Givens
    rotations, stop when |g_{j+1}| <= max(atol, tol |b|) or after `maxiter`
    Arnoldi steps, then x += M (V y).  The call semantics of
    warp.optim.linear.gmres at the reference's call sites
    (tests/test_biharmonic.py:32, tests/test_indefinite.py:130).  Returns
    (x, steps, residual norm, target)."""
    b = np.ascontiguousarray(b, np.float64).reshape(-1)
    n = b.size
    x = np.zeros(n) if x0 is None else np.ascontiguousarray(x0, np.float64).reshape(-1).copy()
    maxiter = maxiter if maxiter > 0 else max(n, 1)
    target = max(atol, tol * np.sqrt(b @ b))
    zero = np.zeros(n)
    op_a = lambda v: A.apply(v, zero, 1.0, 0.0)
    op_m = (lambda v: M.apply(v, zero, 1.0, 0.0)) if M is not None else (lambda v: v.copy())
    m, it = restart, 0
    r = b - op_a(x)
    beta = np.sqrt(r @ r)
    res = beta
    while beta * beta > target * target and np.isfinite(beta) and beta > 0 and it < maxiter:
        V = np.zeros((m + 1, n))
        V[0] = r / beta
        H = np.zeros((m + 1, m))
        cs, sn = np.zeros(m), np.zeros(m)
        g = np.zeros(m + 1)
        g[0] = beta
        k, stop = 0, False
        for j in range(m):
            w = op_a(op_m(V[j]))
            h = V[:j + 1] @ w
            w = w - h @ V[:j + 1]
            h2 = V[:j + 1] @ w
            w = w - h2 @ V[:j + 1]
            h = h + h2
            hn = np.sqrt(w @ w)
            H[:j + 1, j] = h
            H[j + 1, j] = hn
            for i in range(j):
                a_, b_ = H[i, j], H[i + 1, j]
                H[i, j] = cs[i] * a_ + sn[i] * b_
                H[i + 1, j] = -sn[i] * a_ + cs[i] * b_
            a_, b_ = H[j, j], H[j + 1, j]
            c, s_ = 1.0, 0.0
            if b_ != 0.0:
                if abs(b_) > abs(a_):
                    t = a_ / b_
                    s_ = 1.0 / np.sqrt(1.0 + t * t)
                    c = s_ * t
                else:
                    t = b_ / a_
                    c = 1.0 / np.sqrt(1.0 + t * t)
                    s_ = c * t
            cs[j], sn[j] = c, s_
            H[j, j] = c * a_ + s_ * b_
            H[j + 1, j] = 0.0
            g[j + 1] = -s_ * g[j]
            g[j] = c * g[j]
            res = abs(g[j + 1])
            it += 1
            k = j + 1
            stop = res * res <= target * target or it >= maxiter
            if stop or not (hn > 0 and np.isfinite(hn)) or j + 1 == m:
                break
            V[j + 1] = w / hn
        y = np.zeros(k)
        for i in range(k - 1, -1, -1):
            t = g[i] - H[i, i + 1:k] @ y[i + 1:k]
            y[i] = t / H[i, i] if H[i, i] != 0.0 else 0.0
        x = x + op_m(V[:k].T @ y)
        if stop:
            break
        r = b - op_a(x)
        beta = np.sqrt(r @ r)
        res = beta
    return x, it, float(res), float(target)


if os.environ.get("GBPC_ORACLE_THREADS"):
    set_threads(int(os.environ["GBPC_ORACLE_THREADS"]))
