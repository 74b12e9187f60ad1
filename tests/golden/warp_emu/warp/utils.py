"""Array utilities of the Warp emulation (test infrastructure): scans and inner
products over the arrays' scalars."""

from __future__ import annotations

import numpy as np


def array_scan(in_array, out_array, inclusive=True):
    src = in_array.numpy().reshape(-1)
    dst = out_array.numpy().reshape(-1)
    total = np.cumsum(src, dtype=np.int64 if np.issubdtype(src.dtype, np.integer) else src.dtype)
    if inclusive:
        dst[: len(src)] = total
    else:
        dst[0] = 0
        dst[1: len(src)] = total[:-1]


def array_inner(a, b, out=None, count=None, axis=None):
    x = a.numpy().reshape(-1)
    y = b.numpy().reshape(-1)
    acc = x.dtype.type(0)
    for i in range(len(x)):
        acc = acc + x[i] * y[i]
    if out is not None:
        out.numpy()[0] = acc
        return out
    return acc


def array_sum(a, out=None, **k):
    x = a.numpy().reshape(-1)
    acc = x.dtype.type(0)
    for v in x:
        acc = acc + v
    if out is not None:
        out.numpy()[0] = acc
        return out
    return acc
