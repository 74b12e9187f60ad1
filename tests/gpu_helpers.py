"""Shared helpers for the GPU parity tests."""

import numpy as np
import scipy.sparse as ss
import torch


def cuda():
    return torch.device("cuda:0")


def to_bsr(a, dtype=torch.float64, block=1):
    from warp_preconditioners_gb300 import from_scipy

    return from_scipy(ss.csr_matrix(a), cuda(), dtype, (block, block))


def host_csr(m):
    """BsrMatrix (scalar) -> (offsets, columns, values) numpy."""
    return (m.offsets.cpu().numpy(), m.columns.cpu().numpy(), m.values.cpu().numpy())


def vec(x, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x), dtype=dtype, device=cuda()).contiguous()


def oracle_csr(o, a, dtype=np.float64, block=1):
    """The oracle's scalar CSR for the same canonical input the GPU sees."""
    if block == 1:
        c = ss.csr_matrix(a)
        c.sum_duplicates()
        c.sort_indices()
        c.eliminate_zeros()
        return o.CSR(c.indptr, c.indices, c.data.astype(dtype), c.shape[1])
    bsr = ss.bsr_matrix(ss.csr_matrix(a), blocksize=(block, block))
    bsr.sort_indices()
    return o.scalarize(a.shape[0] // block, block, bsr.indptr, bsr.indices, bsr.data.astype(dtype))
