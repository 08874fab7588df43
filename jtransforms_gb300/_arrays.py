"""Array forms accepted by the Java-mirror classes besides flat arrays.

* numpy arrays of any shape, C-contiguous: transformed in place through a
  flat view (the row-major layout of the reference's 1D-array overloads).
* Jagged arrays: nested lists of 1D numpy rows, the counterpart of the
  reference's double[][] / double[][][] overloads (fft/DoubleFFT_2D.java:345,
  fft/DoubleFFT_3D.java:542, dct/DoubleDCT_2D.java:104).  The rows are
  gathered into one contiguous array, transformed, and scattered back.  For
  realForwardFull / realInverseFull the rows are 2 * columns long and only
  their first `columns` values are input (fft/DoubleFFT_2D.java:1010-1021).
"""
from __future__ import annotations

import numpy as np

from . import _native as N


def _rows(a, out):
    if isinstance(a, (list, tuple)):
        for x in a:
            _rows(x, out)
    elif isinstance(a, np.ndarray) and a.ndim == 1:
        out.append(a)
    else:
        raise TypeError("jagged arrays hold 1D numpy rows")
    return out


def run(plan: "N.Plan", op: int, a, offa: int = 0, scale: bool = False):
    if not isinstance(a, (list, tuple)):
        if getattr(a, "ndim", 1) > 1:
            a = a.reshape(-1)  # a view of a C-contiguous array: in place
        return plan.execute(op, a, offa, scale)
    if offa:
        raise N.IllegalArgumentException("jagged arrays take no offset")
    rows = _rows(a, [])
    for r in rows:
        if r.dtype != plan.dtype:
            raise TypeError(f"row dtype {r.dtype} does not match the transform's {np.dtype(plan.dtype)}")
    cols = plan.dims[-1]
    full = plan.kind == N.FFT and op in (N.REAL_FORWARD_FULL, N.REAL_INVERSE_FULL)
    if full:
        # real input in the first `cols` values of each 2 * cols row
        if any(r.size < 2 * cols for r in rows):
            raise N.ArrayIndexOutOfBoundsException("rows of a full real transform hold 2 * columns values")
        buf = np.zeros(2 * len(rows) * cols, plan.dtype)
        buf[: len(rows) * cols] = np.concatenate([r[:cols] for r in rows])
    else:
        buf = np.concatenate(rows)
    plan.execute(op, buf, 0, scale)
    o = 0
    for r in rows:
        n = 2 * cols if full else r.size
        r[:n] = buf[o:o + n]
        o += n
    return a
