"""jtransforms_gb300: JTransforms' transform API on one GB300 GPU.

Classes keep the reference's names, sizes, in-place layouts and exceptions;
every transform runs as sm_103a CUDA kernels in libjtgpu.so (include/jtgpu.h).
There is no CPU fallback: without the library or a GPU the calls raise.
"""
from ._native import (ArrayIndexOutOfBoundsException, IllegalArgumentException,  # noqa: F401
                      IllegalStateException, Plan, launch_count, load)
from .fft import (DoubleFFT_1D, DoubleFFT_2D, DoubleFFT_3D, FloatFFT_1D,  # noqa: F401
                  FloatFFT_2D, FloatFFT_3D)
from .r2r import (DoubleDCT_1D, DoubleDCT_2D, DoubleDCT_3D, DoubleDHT_1D,  # noqa: F401
                  DoubleDHT_2D, DoubleDHT_3D, DoubleDST_1D, DoubleDST_2D,
                  DoubleDST_3D, FloatDCT_1D, FloatDCT_2D, FloatDCT_3D,
                  FloatDHT_1D, FloatDHT_2D, FloatDHT_3D, FloatDST_1D,
                  FloatDST_2D, FloatDST_3D)
from .real_fft_utils import RealFFTUtils_2D, RealFFTUtils_3D  # noqa: F401
from . import utils  # noqa: F401
from .utils import CommonUtils, ConcurrencyUtils  # noqa: F401
