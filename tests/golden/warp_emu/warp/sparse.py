"""Block sparse row matrices of the Warp emulation (test infrastructure).

Restates the documented behaviour of ``warp.sparse`` that the reference relies
on: compact BSR storage (sorted unique block columns per row), assembly from
triplets summing duplicates (all-zero blocks pruned by default), conversion
between block shapes (a block of the new shape is stored when any stored
scalar falls inside it; stored zeros are kept), explicit transposition, and
the product ``y = alpha A x + beta y`` summing each row's blocks in storage
order.
"""

from __future__ import annotations

import numpy as np

from . import types as wt

_wp = None


def _warp():
    global _wp
    if _wp is None:
        import warp

        _wp = warp
    return _wp


class BsrMatrix:
    def __init__(self, nrow, ncol, block_type, device=None):
        wp = _warp()
        self.nrow = int(nrow)
        self.ncol = int(ncol)
        block_type = wt.normalize_dtype(block_type)
        shape = wt.type_shape(block_type)
        self.block_shape = tuple(shape) if shape else (1, 1)
        self.scalar_type = wt.scalar_of(block_type)
        self.dtype = block_type
        self.device = wp.get_device(device)
        self.offsets = wp.zeros(self.nrow + 1, dtype=int, device=self.device)
        self.columns = wp.empty(0, dtype=int, device=self.device)
        self.values = wp.empty(0, dtype=block_type, device=self.device)
        self.row_counts = None

    @property
    def shape(self):
        return (self.nrow * self.block_shape[0], self.ncol * self.block_shape[1])

    @property
    def block_size(self):
        return self.block_shape[0] * self.block_shape[1]

    @property
    def nnz(self):
        return int(self.offsets.numpy()[-1])

    def nnz_sync(self):
        return self.nnz

    def notify_nnz_changed(self, nnz=None):
        """Grow the column and value storage to the count now in the offsets."""
        wp = _warp()
        if nnz is None:
            nnz = int(self.offsets.numpy()[-1])
        if self.columns.shape[0] < nnz:
            self.columns = wp.empty(nnz, dtype=int, device=self.device)
        if self.values.shape[0] < nnz:
            self.values = wp.empty(nnz, dtype=self.dtype, device=self.device)

    @property
    def scalar_values(self):
        return self.values.view(self.scalar_type)

    def uncompress_rows(self):
        off = self.offsets.numpy()
        return np.repeat(np.arange(self.nrow, dtype=np.int32), np.diff(off))

    # host helpers
    def _blocks(self):
        """(rows, cols, values[nnz, b0, b1]) of the stored blocks."""
        nnz = self.nnz
        vals = self.values.numpy()[:nnz].reshape((nnz,) + self.block_shape)
        return self.uncompress_rows(), self.columns.numpy()[:nnz].copy(), vals

    def __matmul__(self, x):
        return bsr_mv(self, x)


def _block_type(block_shape, scalar_type):
    if tuple(block_shape) == (1, 1):
        return scalar_type
    return wt.matrix(tuple(block_shape), scalar_type)


def _from_sorted_blocks(nrow, ncol, rows, cols, vals, block_shape, scalar_type, device):
    wp = _warp()
    out = BsrMatrix(nrow, ncol, _block_type(block_shape, scalar_type), device)
    counts = np.bincount(rows, minlength=nrow) if len(rows) else np.zeros(nrow, np.int64)
    off = np.zeros(nrow + 1, dtype=np.int32)
    np.cumsum(counts, out=off[1:])
    out.offsets = wp.array(off, dtype=int, device=out.device)
    out.columns = wp.array(np.asarray(cols, dtype=np.int32), dtype=int, device=out.device)
    v = np.asarray(vals, dtype=scalar_type)
    if tuple(block_shape) == (1, 1):
        v = v.reshape(-1)
    else:
        v = v.reshape((-1,) + tuple(block_shape))
    out.values = wp.array(dtype=out.dtype, device=out.device, _buffer=v.copy())
    return out


def _assemble(nrow, ncol, rows, cols, vals, block_shape, scalar_type, device, prune):
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    vals = np.asarray(vals, dtype=scalar_type).reshape((-1,) + tuple(block_shape))
    if rows.size == 0:
        return _from_sorted_blocks(nrow, ncol, rows, cols, vals, block_shape, scalar_type, device)
    keys = rows * ncol + cols
    order = np.argsort(keys, kind="stable")
    keys_s = keys[order]
    uniq, start = np.unique(keys_s, return_index=True)
    summed = np.zeros((len(uniq),) + tuple(block_shape), dtype=scalar_type)
    # duplicates summed in their input order
    seg = np.searchsorted(uniq, keys_s)
    for k in range(len(order)):
        summed[seg[k]] = summed[seg[k]] + vals[order[k]]
    urows = (uniq // ncol).astype(np.int64)
    ucols = (uniq % ncol).astype(np.int64)
    if prune:
        keep = np.any(summed.reshape(len(uniq), -1) != 0, axis=1)
        urows, ucols, summed = urows[keep], ucols[keep], summed[keep]
    return _from_sorted_blocks(nrow, ncol, urows, ucols, summed, block_shape, scalar_type,
                               device)


def bsr_zeros(rows_of_blocks, cols_of_blocks, block_type, device=None):
    return BsrMatrix(rows_of_blocks, cols_of_blocks, block_type, device)


def bsr_from_triplets(rows_of_blocks, cols_of_blocks, rows, columns, values,
                      prune_numerical_zeros=True, masked=False, device=None):
    block_type = values.dtype
    shape = wt.type_shape(block_type) or (1, 1)
    return _assemble(rows_of_blocks, cols_of_blocks, rows.numpy(), columns.numpy(),
                     values.numpy(), shape, wt.scalar_of(block_type), values.device,
                     prune_numerical_zeros)


def bsr_set_from_triplets(dest, rows, columns, values, prune_numerical_zeros=True, masked=False):
    out = bsr_from_triplets(dest.nrow, dest.ncol, rows, columns, values, prune_numerical_zeros)
    dest.offsets, dest.columns, dest.values = out.offsets, out.columns, out.values
    return dest


def bsr_copy(A, scalar_type=None, block_shape=None, structure_only=False):
    scalar_type = wt.normalize_dtype(scalar_type) if scalar_type is not None else A.scalar_type
    block_shape = tuple(block_shape) if block_shape is not None else A.block_shape
    rows, cols, vals = A._blocks()
    b0, b1 = A.block_shape
    if block_shape == A.block_shape:
        return _from_sorted_blocks(A.nrow, A.ncol, rows, cols, vals.astype(scalar_type),
                                   block_shape, scalar_type, A.device)
    # scalar triplets of every stored entry (zeros included), regrouped
    n = len(rows)
    ii, jj = np.meshgrid(np.arange(b0), np.arange(b1), indexing="ij")
    srow = (rows[:, None, None] * b0 + ii[None]).reshape(-1)
    scol = (cols[:, None, None] * b1 + jj[None]).reshape(-1)
    sval = vals.reshape(n * b0 * b1)
    c0, c1 = block_shape
    nrow = A.nrow * b0 // c0
    ncol = A.ncol * b1 // c1
    brow, bcol = srow // c0, scol // c1
    keys = brow.astype(np.int64) * ncol + bcol
    uniq, inv = np.unique(keys, return_inverse=True)
    out_vals = np.zeros((len(uniq), c0, c1), dtype=scalar_type)
    out_vals[inv, srow % c0, scol % c1] = sval.astype(scalar_type)
    return _from_sorted_blocks(nrow, ncol, uniq // ncol, uniq % ncol, out_vals, block_shape,
                               scalar_type, A.device)


def bsr_transposed(A):
    rows, cols, vals = A._blocks()
    order = np.lexsort((rows, cols))
    tv = np.swapaxes(vals[order], 1, 2)
    bs = (A.block_shape[1], A.block_shape[0])
    return _from_sorted_blocks(A.ncol, A.nrow, cols[order], rows[order], tv, bs, A.scalar_type,
                               A.device)


def _as_blocks(arr, b):
    flat = arr.numpy().reshape(-1)
    return flat.reshape(-1, b)


def bsr_mv(A, x, y=None, alpha=1.0, beta=0.0, transpose=False, work_buffer=None):
    wp = _warp()
    if transpose:
        A = bsr_transposed(A)
    b0, b1 = A.block_shape
    st = A.scalar_type
    if y is None:
        y = wp.zeros(A.nrow * b0 if x.dtype == st else A.nrow, dtype=x.dtype, device=A.device)
        beta = 0.0
    xs = _as_blocks(x, b1).astype(st, copy=False)
    ys = _as_blocks(y, b0)
    off = A.offsets.numpy()
    col = A.columns.numpy()
    nnz = A.nnz
    vals = A.values.numpy()[:nnz].reshape(nnz, b0, b1)
    lengths = np.diff(off)
    acc = np.zeros((A.nrow, b0), dtype=st)
    with np.errstate(all="ignore"):
        # alpha == 0 never reads x (NaNs there do not reach y)
        for k in range(int(lengths.max()) if A.nrow and alpha != 0.0 else 0):
            rows = np.flatnonzero(lengths > k)
            e = off[rows] + k
            blk = vals[e]
            xv = xs[col[e]]
            prod = blk[:, :, 0] * xv[:, 0:1]
            for j in range(1, b1):
                prod = prod + blk[:, :, j] * xv[:, j:j + 1]
            acc[rows] = acc[rows] + prod
        out = st(alpha) * acc
        if beta != 0.0:
            out = out + st(beta) * ys
    ys[...] = out
    return y
