"""Accessors for the packed output of 2D/3D realForward
(org.jtransforms.fft.RealFFTUtils_2D / RealFFTUtils_3D).

DoubleFFT_2D/3D.realForward (and the Float twins) leave half of the
Hermitian spectrum of real data in the input array, in a packed layout
(fft/DoubleFFT_2D.java:788-815, fft/DoubleFFT_3D.java:1290-1336).  These
classes give callers the full-spectrum view of that array without unpacking
it: mode [r][c] (2D) or [s][r][c] (3D), where an even c is the real part and
an odd c the imaginary part of Fourier mode c // 2, c in [0, 2 * columns),
the indexing of realForwardFull's output.

    getIndex(r, c) / getIndex(s, r, c)
        index >= 0   the mode is packed[index]
        index < 0    the mode is -packed[-index]
        ZERO         the mode is always zero (the imaginary part of a
                     self-conjugate mode)
    pack(val, r, c, packed[, pos])      writes mode [r][c]; a mode that is
                                        always zero raises IllegalArgumentException
    unpack(r, c, packed[, pos])         reads mode [r][c]

`packed` is a flat numpy array or CUDA tensor (the double[]/float[] and
LargeArray overloads, `pos` = offset of the first element), or a jagged
array: a list of row arrays (2D, the double[][] overloads) or a list of
lists of row arrays (3D, double[][][]).  ZERO is Java's Integer.MIN_VALUE
when every index fits in an int and Long.MIN_VALUE otherwise, like the
reference's int and long overloads.

The slot of each mode follows from the packed layout and Hermitian symmetry
F[k] = conj(F[-k]); the reference's classes (fft/RealFFTUtils_2D.java:159-666,
fft/RealFFTUtils_3D.java:192-794) define the same mapping.  The 2D layout is
the 3D one with a single slice.
"""
from __future__ import annotations

from ._native import IllegalArgumentException

INT_MIN = -(1 << 31)
LONG_MIN = -(1 << 63)


def _locate(S, R, C, k1, k2, c):
    """(index, sign) of component c of mode [k1][k2][c // 2] in the packed
    layout of an S x R x C real transform; sign 0 means always zero."""
    k3, im = c >> 1, c & 1
    flip = 1
    SS, RS = R * C, C
    if k3 > C // 2:
        # F[k1][k2][k3] = conj(F[-k1][-k2][C - k3])
        k1, k2, k3 = (S - k1) % S, (R - k2) % R, C - k3
        flip = -1 if im else 1
    if 0 < k3 < C // 2:
        return k1 * SS + k2 * RS + 2 * k3 + im, flip
    h = k3 == C // 2  # the column-C/2 modes share slots with column 0
    if k2 != 0 and 2 * k2 != R:
        if not h:
            if 2 * k2 < R:
                return k1 * SS + k2 * RS + im, flip
            base = ((S - k1) % S) * SS + (R - k2) * RS
            return (base, flip) if not im else (base + 1, -flip)
        if 2 * k2 > R:
            base = k1 * SS + k2 * RS
            return (base + 1, flip) if not im else (base, flip)
        base = ((S - k1) % S) * SS + (R - k2) * RS
        return (base + 1, flip) if not im else (base, -flip)
    rb = k2 * RS  # row 0 or R/2
    if k1 == 0 or 2 * k1 == S:
        return (k1 * SS + rb + (1 if h else 0), flip) if not im else (0, 0)
    if not h:
        if 2 * k1 < S:
            return k1 * SS + rb + im, flip
        base = (S - k1) * SS + rb
        return (base, flip) if not im else (base + 1, -flip)
    if 2 * k1 < S:
        base = (S - k1) * SS + rb
        return (base + 1, flip) if not im else (base, -flip)
    base = k1 * SS + rb
    return (base + 1, flip) if not im else (base, flip)


class _PackedAccess:
    def __init__(self, dims):
        self._S, self._R, self._C = dims
        self.ZERO = INT_MIN if self._S * self._R * self._C < (1 << 31) else LONG_MIN

    def _index(self, k1, k2, c):
        S, R, C = self._S, self._R, self._C
        if not (0 <= k1 < S and 0 <= k2 < R and 0 <= c < 2 * C):
            raise IndexError(f"mode [{k1}][{k2}][{c}] outside {S} x {R} x {2 * C}")
        idx, sgn = _locate(S, R, C, k1, k2, c)
        if sgn == 0:
            return self.ZERO
        return idx if sgn > 0 else -idx

    def _get(self, packed, i, pos):
        if isinstance(packed, (list, tuple)):
            row, col = self._jagged(i)
            return row(packed)[col]
        return packed[pos + i]

    def _set(self, packed, i, pos, val):
        if isinstance(packed, (list, tuple)):
            row, col = self._jagged(i)
            row(packed)[col] = val
        else:
            packed[pos + i] = val

    def _unpack(self, idx, packed, pos):
        if idx == self.ZERO:
            return 0.0
        return self._get(packed, idx, pos) if idx >= 0 else -self._get(packed, -idx, pos)

    def _pack(self, val, idx, packed, pos, where):
        if idx == self.ZERO:
            raise IllegalArgumentException(f"{where} component cannot be modified (always zero)")
        if idx >= 0:
            self._set(packed, idx, pos, val)
        else:
            self._set(packed, -idx, pos, -val)


class RealFFTUtils_2D(_PackedAccess):
    """fft/RealFFTUtils_2D.java: access to DoubleFFT_2D / FloatFFT_2D
    realForward output as the rows x 2*columns full spectrum."""

    def __init__(self, rows: int, columns: int):
        super().__init__((1, int(rows), int(columns)))
        self.rows, self.columns = int(rows), int(columns)

    def getIndex(self, r: int, c: int) -> int:
        return self._index(0, int(r), int(c))

    def _jagged(self, i):
        return (lambda p: p[i // self.columns]), i % self.columns

    def pack(self, val, r: int, c: int, packed, pos: int = 0):
        self._pack(val, self.getIndex(r, c), packed, pos, f"[{r}][{c}]")

    def unpack(self, r: int, c: int, packed, pos: int = 0):
        return self._unpack(self.getIndex(r, c), packed, pos)


class RealFFTUtils_3D(_PackedAccess):
    """fft/RealFFTUtils_3D.java: access to DoubleFFT_3D / FloatFFT_3D
    realForward output as the slices x rows x 2*columns full spectrum
    (sliceStride = rows * columns, rowStride = columns in the packed array)."""

    def __init__(self, slices: int, rows: int, columns: int):
        super().__init__((int(slices), int(rows), int(columns)))
        self.slices, self.rows, self.columns = int(slices), int(rows), int(columns)
        self.rowStride = self.columns
        self.sliceStride = self.rows * self.columns

    def getIndex(self, s: int, r: int, c: int) -> int:
        return self._index(int(s), int(r), int(c))

    def _jagged(self, i):
        s, rem = divmod(i, self.sliceStride)
        r, col = divmod(rem, self.rowStride)
        return (lambda p: p[s][r]), col

    def pack(self, val, s: int, r: int, c: int, packed, pos: int = 0):
        self._pack(val, self.getIndex(s, r, c), packed, pos, f"[{s}][{r}][{c}]")

    def unpack(self, s: int, r: int, c: int, packed, pos: int = 0):
        return self._unpack(self.getIndex(s, r, c), packed, pos)
