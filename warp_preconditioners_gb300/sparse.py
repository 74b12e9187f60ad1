"""Block sparse matrices carried by torch tensors.

`BsrMatrix` mirrors the fields the reference reads from ``warp.sparse.BsrMatrix``
(``offsets``, ``columns``, ``values``, ``block_shape``, ``nrow``, ``ncol``,
``shape``, ``scalar_type``, ``nnz``, ``row_counts``, ``nnz_sync()``) so that the
preconditioner constructors read like the reference's.  Storage is always
compact and canonical: sorted, unique block columns per row.  Values are a
tensor of shape ``[nnz]`` for 1 x 1 blocks and ``[nnz, b, b]`` otherwise.

Format conversions that the reference delegates to warp.sparse (scalarise,
transpose, scalar-to-block) run as libgbpc kernels; assembling from triplets
(the role of ``bsr_from_triplets``) is data-format plumbing done with torch
sorting on the tensors' own device.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib


class BsrMatrix:
    def __init__(self, nrow, ncol, block_shape, offsets, columns, values):
        self.nrow = int(nrow)
        self.ncol = int(ncol)
        self.block_shape = tuple(int(b) for b in block_shape)
        self.offsets = offsets
        self.columns = columns
        self.values = values
        self.row_counts = None  # always compact

    @property
    def block_size(self) -> int:
        return self.block_shape[0] * self.block_shape[1]

    @property
    def shape(self):
        return (self.nrow * self.block_shape[0], self.ncol * self.block_shape[1])

    @property
    def scalar_type(self) -> torch.dtype:
        return self.values.dtype

    @property
    def dtype(self) -> torch.dtype:
        return self.values.dtype

    @property
    def device(self) -> torch.device:
        return self.values.device

    @property
    def nnz(self) -> int:
        return int(self.columns.numel())

    def nnz_sync(self) -> int:
        return self.nnz

    def scalar_values(self) -> torch.Tensor:
        """Values as a flat tensor of scalars (block-major, row-major blocks)."""
        return self.values.reshape(-1)

    def to_scipy(self):
        import scipy.sparse as ss

        b = self.block_shape[0]
        off = self.offsets.cpu().numpy()
        col = self.columns.cpu().numpy()
        val = self.values.detach().to(torch.float64).cpu().numpy()
        if b == 1:
            return ss.csr_matrix((val.reshape(-1), col, off), shape=self.shape)
        return ss.bsr_matrix((val.reshape(-1, b, b), col, off), shape=self.shape).tocsr()

    def dense(self) -> np.ndarray:
        return self.to_scipy().toarray()


def _device(device) -> torch.device:
    return torch.device(device) if device is not None else torch.device("cuda")


def bsr_from_triplets(nrow, ncol, rows, cols, values, prune_numerical_zeros=True):
    """Assemble compact BSR from (possibly repeated) block triplets, summing duplicates."""
    rows = torch.as_tensor(rows).to(torch.int64)
    cols = torch.as_tensor(cols, device=rows.device).to(torch.int64)
    values = torch.as_tensor(values, device=rows.device)
    if values.dim() == 1:
        block_shape = (1, 1)
    else:
        block_shape = tuple(values.shape[1:])
    keys = rows * int(ncol) + cols
    uniq, inverse = torch.unique(keys, sorted=True, return_inverse=True)
    summed = torch.zeros((uniq.numel(),) + tuple(values.shape[1:]), dtype=values.dtype,
                         device=values.device)
    summed.index_add_(0, inverse, values)
    if prune_numerical_zeros:
        flat = summed.reshape(summed.shape[0], -1)
        keep = (flat != 0).any(dim=1)
        uniq, summed = uniq[keep], summed[keep]
    r = (uniq // int(ncol)).to(torch.int64)
    c = (uniq % int(ncol)).to(torch.int32)
    counts = torch.bincount(r, minlength=int(nrow))
    offsets = torch.zeros(int(nrow) + 1, dtype=torch.int64, device=values.device)
    offsets[1:] = torch.cumsum(counts, 0)
    return BsrMatrix(nrow, ncol, block_shape, offsets.to(torch.int32).contiguous(), c.contiguous(),
                     summed.contiguous())


def from_scipy(a, device=None, dtype=torch.float64, block_shape=(1, 1)) -> BsrMatrix:
    """Canonical BSR from a SciPy sparse or dense matrix (host -> device upload)."""
    import scipy.sparse as ss

    dev = _device(device)
    b = block_shape[0]
    if b == 1:
        c = ss.csr_matrix(a)
        c.sum_duplicates()
        c.sort_indices()
        c.eliminate_zeros()
        return BsrMatrix(
            c.shape[0], c.shape[1], (1, 1),
            torch.as_tensor(c.indptr.astype(np.int32), device=dev),
            torch.as_tensor(c.indices.astype(np.int32), device=dev),
            torch.as_tensor(c.data, dtype=dtype, device=dev),
        )
    bsr = ss.bsr_matrix(ss.csr_matrix(a), blocksize=(b, b))
    bsr.sum_duplicates()
    bsr.sort_indices()
    return BsrMatrix(
        bsr.shape[0] // b, bsr.shape[1] // b, (b, b),
        torch.as_tensor(bsr.indptr.astype(np.int32), device=dev),
        torch.as_tensor(bsr.indices.astype(np.int32), device=dev),
        torch.as_tensor(bsr.data, dtype=dtype, device=dev),
    )


def scalarize(a: BsrMatrix) -> BsrMatrix:
    """b x b BSR to scalar CSR keeping stored zeros (fsai_pack.py:74-130)."""
    b = a.block_shape[0]
    if b == 1:
        return a
    n = a.nrow * b
    dev = a.device
    out_off = torch.empty(n + 1, dtype=torch.int32, device=dev)
    out_col = torch.empty(a.nnz * b * b, dtype=torch.int32, device=dev)
    out_val = torch.empty(a.nnz * b * b, dtype=a.scalar_type, device=dev)
    _lib.call("gbpc_scalarize", a.nrow, b, _lib.ptr(a.offsets), _lib.ptr(a.columns),
              _lib.ptr(a.values), _lib.dtype_code(a.scalar_type), _lib.ptr(out_off),
              _lib.ptr(out_col), _lib.ptr(out_val), _lib.stream(dev))
    return BsrMatrix(n, a.ncol * b, (1, 1), out_off, out_col, out_val)


def to_blocks(a: BsrMatrix, b: int) -> BsrMatrix:
    """Scalar CSR (rows grouped by b) to b x b BSR, zero-filling stored blocks."""
    if a.block_shape != (1, 1):
        raise ValueError("to_blocks expects a scalar matrix")
    if b == 1:
        return a
    if a.nrow % b or a.ncol % b:
        raise ValueError("matrix size is not a multiple of the block size")
    nb = a.nrow // b
    dev = a.device
    boff = torch.empty(nb + 1, dtype=torch.int32, device=dev)
    nnzb = ctypes.c_int64()
    code = _lib.dtype_code(a.scalar_type)
    _lib.call("gbpc_csr_to_bsr", nb, b, _lib.ptr(a.offsets), _lib.ptr(a.columns),
              _lib.ptr(a.values), code, _lib.ptr(boff), None, None, ctypes.byref(nnzb),
              _lib.stream(dev))
    bcol = torch.empty(nnzb.value, dtype=torch.int32, device=dev)
    bval = torch.empty((nnzb.value, b, b), dtype=a.scalar_type, device=dev)
    _lib.call("gbpc_csr_to_bsr", nb, b, _lib.ptr(a.offsets), _lib.ptr(a.columns),
              _lib.ptr(a.values), code, _lib.ptr(boff), _lib.ptr(bcol), _lib.ptr(bval),
              ctypes.byref(nnzb), _lib.stream(dev))
    return BsrMatrix(nb, a.ncol // b, (b, b), boff, bcol, bval)


def bsr_copy(a: BsrMatrix, block_shape=None, scalar_type=None) -> BsrMatrix:
    """Copy with an optional block-shape or scalar-type change."""
    out = a
    if block_shape is not None and tuple(block_shape) != a.block_shape:
        if tuple(block_shape) == (1, 1):
            out = scalarize(a)
        elif a.block_shape == (1, 1):
            out = to_blocks(a, block_shape[0])
        else:
            out = to_blocks(scalarize(a), block_shape[0])
    else:
        out = BsrMatrix(a.nrow, a.ncol, a.block_shape, a.offsets.clone(), a.columns.clone(),
                        a.values.clone())
    if scalar_type is not None and scalar_type != out.scalar_type:
        out = BsrMatrix(out.nrow, out.ncol, out.block_shape, out.offsets, out.columns,
                        out.values.to(scalar_type))
    return out


def bsr_transposed(a: BsrMatrix) -> BsrMatrix:
    """Explicit transpose (blocks transposed too)."""
    b = a.block_shape[0]
    dev = a.device
    t_off = torch.empty(a.ncol + 1, dtype=torch.int32, device=dev)
    t_col = torch.empty(a.nnz, dtype=torch.int32, device=dev)
    t_val = torch.empty_like(a.values)
    code = _lib.dtype_code(a.scalar_type)
    if b == 1:
        _lib.call("gbpc_csr_transpose", a.nrow, a.ncol, _lib.ptr(a.offsets), _lib.ptr(a.columns),
                  _lib.ptr(a.values), code, _lib.ptr(t_off), _lib.ptr(t_col), _lib.ptr(t_val),
                  _lib.stream(dev))
    else:
        _lib.call("gbpc_bsr_transpose", a.nrow, a.ncol, b, _lib.ptr(a.offsets),
                  _lib.ptr(a.columns), _lib.ptr(a.values), code, _lib.ptr(t_off),
                  _lib.ptr(t_col), _lib.ptr(t_val), _lib.stream(dev))
    return BsrMatrix(a.ncol, a.nrow, (b, b), t_off, t_col, t_val)


def bsr_mv(a: BsrMatrix, x, y, alpha=1.0, beta=0.0):
    """y = alpha * A x + beta * y (warp.sparse.bsr_mv semantics)."""
    from .linear import aslinearoperator

    aslinearoperator(a).matvec(x, y, y, alpha, beta)
    return y


def spgemm(A: BsrMatrix, B: BsrMatrix, col_scale=None, add_diag=None) -> BsrMatrix:
    """``A diag(col_scale) B + diag(add_diag)`` on the device (float64 scalar
    CSR): the host SciPy assembly ``A @ diags(d) @ B + diags(e)`` with the
    same summation order (with ``col_scale``, over the inner index downwards,
    as SciPy's intermediate ``A @ diags(d)`` stores its rows; without it,
    upwards, as ``A @ B``), exact zeros dropped and rows sorted."""
    import ctypes

    from . import _lib

    for m in (A, B):
        if m.block_shape != (1, 1) or m.scalar_type != torch.float64:
            raise ValueError("spgemm takes float64 scalar CSR matrices")
    if A.ncol != B.nrow:
        raise ValueError("inner dimensions differ")
    dev = A.device
    if col_scale is not None and (col_scale.dtype != torch.float64 or col_scale.numel() != A.ncol):
        raise ValueError("col_scale must be float64 with one entry per column of A")
    if add_diag is not None and (add_diag.dtype != torch.float64 or add_diag.numel() != A.nrow
                                 or A.nrow > B.ncol):
        raise ValueError("add_diag must be float64 with one entry per row")
    d = col_scale.contiguous() if col_scale is not None else None
    e = add_diag.contiguous() if add_diag is not None else None
    off = torch.empty(A.nrow + 1, dtype=torch.int32, device=dev)
    nnz = ctypes.c_int64()
    args = [A.nrow, B.ncol, _lib.ptr(A.offsets), _lib.ptr(A.columns), _lib.ptr(A.values),
            _lib.ptr(d) if d is not None else None, B.nrow, _lib.ptr(B.offsets),
            _lib.ptr(B.columns), _lib.ptr(B.values), _lib.ptr(e) if e is not None else None,
            _lib.ptr(off)]
    _lib.call("gbpc_spgemm", *args, None, None, ctypes.byref(nnz), _lib.stream(dev))
    col = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=dev)
    val = torch.empty(max(nnz.value, 1), dtype=torch.float64, device=dev)
    _lib.call("gbpc_spgemm", *args, _lib.ptr(col), _lib.ptr(val), ctypes.byref(nnz),
              _lib.stream(dev))
    return BsrMatrix(A.nrow, B.ncol, (1, 1), off, col[:nnz.value], val[:nnz.value])


def block_diag(mats) -> BsrMatrix:
    """Block-diagonal concatenation of BSR matrices with the same block shape
    and dtype (the systems of a multi-system solve): row offsets and
    columns shifted, values concatenated; canonical when each input is."""
    mats = list(mats)
    if not mats:
        raise ValueError("block_diag needs at least one matrix")
    bs, dt, dev = mats[0].block_shape, mats[0].scalar_type, mats[0].device
    for m in mats:
        if m.block_shape != bs or m.scalar_type != dt or m.device != dev:
            raise ValueError("block_diag needs one block shape, dtype and device")
    offs, cols, vals = [torch.zeros(1, dtype=torch.int32, device=dev)], [], []
    row0 = col0 = nz0 = 0
    for m in mats:
        offs.append(m.offsets[1:].to(torch.int64) + nz0)
        cols.append(m.columns.to(torch.int64) + col0)
        vals.append(m.values)
        row0 += m.nrow
        col0 += m.ncol
        nz0 += m.nnz
    if nz0 > 0x7fffffff or col0 > 0x7fffffff:
        raise ValueError("block_diag result exceeds 32-bit indices")
    off = torch.cat([o.to(torch.int32) for o in offs])
    col = torch.cat(cols).to(torch.int32) if cols else torch.zeros(0, dtype=torch.int32, device=dev)
    val = torch.cat(vals)
    return BsrMatrix(row0, col0, bs, off, col, val)
