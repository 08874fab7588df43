"""FFT classes with JTransforms' Java API (org.jtransforms.fft).

Each class mirrors its Java namesake: the constructor takes the sizes and
validates them like the reference, and every method transforms the caller's
array in place with the reference's layouts.  Arrays are numpy arrays (host;
copied to the GPU and back per call) or CUDA torch tensors (device-resident).
Java overloads map to optional arguments:

    complexForward(a) / complexForward(a, offa)
    complexInverse(a, scale) / complexInverse(a, offa, scale)
    realForward(a) / realForward(a, offa)
    realForwardFull(a) / realForwardFull(a, offa)
    realInverse(a, scale) / realInverse(a, offa, scale)
    realInverseFull(a, scale) / realInverseFull(a, offa, scale)

Reference: fft/DoubleFFT_1D.java:117-1422, fft/FloatFFT_1D.java,
fft/DoubleFFT_2D.java, fft/FloatFFT_2D.java, fft/DoubleFFT_3D.java,
fft/FloatFFT_3D.java (src/main/java/org/jtransforms/).
"""
from __future__ import annotations

from . import _arrays
from . import _native as N
from ._native import IllegalArgumentException


def _off_scale(args, name):
    if len(args) == 1:
        return 0, bool(args[0])
    if len(args) == 2:
        return int(args[0]), bool(args[1])
    raise TypeError(f"{name}(a, [offa,] scale)")


class _FFTBase:
    _prec = N.FLOAT64

    def __init__(self, *dims):
        self._plan = N.Plan(N.FFT, self._prec, dims)

    def _run(self, op, a, offa=0, scale=False):
        return _arrays.run(self._plan, op, a, offa, scale)

    # Java methods -----------------------------------------------------
    def complexForward(self, a, offa: int = 0):
        """Forward DFT of complex data in place: a[offa+2k]=Re, a[offa+2k+1]=Im
        (fft/DoubleFFT_1D.java:243)."""
        self._run(N.COMPLEX_FORWARD, a, offa)

    def complexInverse(self, a, *args):
        """Inverse DFT of complex data; scale=True multiplies by 1/n
        (fft/DoubleFFT_1D.java:362)."""
        offa, scale = _off_scale(args, "complexInverse")
        self._run(N.COMPLEX_INVERSE, a, offa, scale)

    def realForward(self, a, offa: int = 0):
        """Forward DFT of real data, packed half spectrum (fft/DoubleFFT_1D.java:524)."""
        self._run(N.REAL_FORWARD, a, offa)

    def realForwardFull(self, a, offa: int = 0):
        """Forward DFT of n reals into the full 2n-slot complex spectrum
        (fft/DoubleFFT_1D.java:678)."""
        self._run(N.REAL_FORWARD_FULL, a, offa)

    def realInverse(self, a, *args):
        """Inverse of realForward (fft/DoubleFFT_1D.java:946).  Unscaled, the
        result is n/2 * x for power-of-two n and n * x otherwise, as in the
        reference."""
        offa, scale = _off_scale(args, "realInverse")
        self._run(N.REAL_INVERSE, a, offa, scale)

    def realInverseFull(self, a, *args):
        """Inverse DFT of n reals into the full 2n-slot complex result
        (fft/DoubleFFT_1D.java:1112)."""
        offa, scale = _off_scale(args, "realInverseFull")
        self._run(N.REAL_INVERSE_FULL, a, offa, scale)

    # extensions -------------------------------------------------------
    @property
    def plan(self) -> N.Plan:
        return self._plan


class DoubleFFT_1D(_FFTBase):
    """fft/DoubleFFT_1D.java: 1D FFT of double data, n >= 1."""
    _prec = N.FLOAT64

    def __init__(self, n: int):
        if n < 1:
            raise IllegalArgumentException("n must be greater than 0")
        super().__init__(n)


class FloatFFT_1D(DoubleFFT_1D):
    """fft/FloatFFT_1D.java: 1D FFT of float data."""
    _prec = N.FLOAT32


class DoubleFFT_2D(_FFTBase):
    """fft/DoubleFFT_2D.java: 2D FFT, row-major rows x columns, both > 1.
    realForward/realInverse need power-of-two sizes (packed layout of
    fft/DoubleFFT_2D.java:788-815)."""
    _prec = N.FLOAT64

    def __init__(self, rows: int, columns: int):
        if rows <= 1 or columns <= 1:
            raise IllegalArgumentException("rows and columns must be greater than 1")
        super().__init__(rows, columns)


class FloatFFT_2D(DoubleFFT_2D):
    """fft/FloatFFT_2D.java."""
    _prec = N.FLOAT32


class DoubleFFT_3D(_FFTBase):
    """fft/DoubleFFT_3D.java: 3D FFT, slices x rows x columns, each > 1;
    complex layout a[s*2*rows*cols + r*2*cols + 2c (+1)]."""
    _prec = N.FLOAT64

    def __init__(self, slices: int, rows: int, columns: int):
        if slices <= 1 or rows <= 1 or columns <= 1:
            raise IllegalArgumentException("slices, rows and columns must be greater than 1")
        super().__init__(slices, rows, columns)


class FloatFFT_3D(DoubleFFT_3D):
    """fft/FloatFFT_3D.java."""
    _prec = N.FLOAT32
