"""RealFFTUtils_2D / RealFFTUtils_3D (fft/RealFFTUtils_2D.java:159-666,
fft/RealFFTUtils_3D.java:192-794): reading and writing the packed output of
2D/3D realForward as the full spectrum.

CPU tests read the oracle's packed output (its 3D layout is pinned to the
reference test's fillSymmetric) and compare every mode with numpy's FP64
FFT of the same input; the GPU test does the same on the library's own
realForward output.  Tolerance: 1e-12 of the spectrum's largest magnitude
(double), 4 * eps_float * log2(N) relative L2 (float GPU output)."""
import numpy as np
import pytest

import jtransforms_gb300 as J
from tests._helpers import rel_l2, tol

SHAPES_2D = [(2, 2), (2, 8), (8, 2), (4, 8), (16, 16), (8, 32)]
SHAPES_3D = [(2, 2, 2), (2, 4, 8), (4, 4, 4), (8, 2, 4), (4, 8, 16), (16, 8, 2)]


def _full(shape, packed, util):
    """The full rows x 2*columns spectrum read through the accessor."""
    cols = shape[-1]
    out = np.zeros(shape[:-1] + (2 * cols,))
    for idx in np.ndindex(*out.shape):
        out[idx] = util.unpack(*idx, packed)
    return out


def _want(x):
    f = np.fft.fftn(x)
    w = np.empty(x.shape[:-1] + (2 * x.shape[-1],))
    w[..., 0::2] = f.real
    w[..., 1::2] = f.imag
    return w


def _util(shape):
    return J.RealFFTUtils_2D(*shape) if len(shape) == 2 else J.RealFFTUtils_3D(*shape)


@pytest.mark.parametrize("shape", SHAPES_2D + SHAPES_3D)
def test_unpack_pack_match_full_spectrum(oracle, shape):
    rng = np.random.default_rng(sum(shape))
    x = rng.uniform(-1, 1, shape)
    packed = x.ravel().copy()
    oracle.run(oracle.FFT, oracle.REAL_FORWARD, list(shape), packed)
    util = _util(shape)
    want = _want(x)
    got = _full(shape, packed, util)
    assert np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want))
    # the modes reported as always zero are the imaginary parts of the
    # self-conjugate modes, and only those
    zero = np.zeros(want.shape, bool)
    for idx in np.ndindex(*want.shape):
        zero[idx] = util.getIndex(*idx) == util.ZERO
    k = [np.arange(n) for n in shape]
    grids = np.meshgrid(*k, indexing="ij")
    selfconj = np.ones(shape, bool)
    for g, n in zip(grids, shape):
        selfconj &= (g == 0) | (2 * g == n)
    expect = np.zeros(want.shape, bool)
    expect[..., 1::2] = selfconj
    assert np.array_equal(zero, expect)
    # writing every mode of the full spectrum rebuilds the packed array
    rebuilt = np.full_like(packed, np.nan)
    for idx in np.ndindex(*want.shape):
        if util.getIndex(*idx) != util.ZERO:
            util.pack(want[idx], *idx, rebuilt)
    assert np.max(np.abs(rebuilt - packed)) <= 1e-12 * np.max(np.abs(want))
    # an offset array and the jagged (double[][] / double[][][]) forms
    off = np.concatenate([np.zeros(3), packed])
    jag = [r.copy() for r in packed.reshape(-1, shape[-1])]
    if len(shape) == 3:
        jag = [jag[s * shape[1]:(s + 1) * shape[1]] for s in range(shape[0])]
    for idx in list(np.ndindex(*want.shape))[:: max(1, want.size // 97)]:
        assert util.unpack(*idx, off, 3) == util.unpack(*idx, packed)
        assert util.unpack(*idx, jag) == util.unpack(*idx, packed)


def test_always_zero_modes_cannot_be_written():
    u = J.RealFFTUtils_2D(4, 8)
    a = np.zeros(32)
    assert u.getIndex(0, 1) == u.ZERO == -(1 << 31)
    with pytest.raises(J.IllegalArgumentException):
        u.pack(1.0, 0, 1, a)
    u.pack(0.0, 0, 0, a)
    v = J.RealFFTUtils_3D(2, 4, 8)
    with pytest.raises(J.IllegalArgumentException):
        v.pack(1.0, 1, 2, 9, np.zeros(64))
    with pytest.raises(IndexError):
        u.unpack(4, 0, a)
    assert J.RealFFTUtils_2D(1 << 16, 1 << 16).ZERO == -(1 << 63)  # LargeArray-sized: long indices


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("shape", [(16, 32), (64, 8), (8, 16, 32), (16, 4, 8)])
def test_gpu_real_forward_read_through_accessor(prec, shape):
    dt = np.float64 if prec == "f64" else np.float32
    N = int(np.prod(shape))
    x = np.random.default_rng(N).uniform(-1, 1, shape)
    a = x.ravel().astype(dt)
    cls = {(2, "f64"): J.DoubleFFT_2D, (2, "f32"): J.FloatFFT_2D,
           (3, "f64"): J.DoubleFFT_3D, (3, "f32"): J.FloatFFT_3D}[(len(shape), prec)]
    cls(*shape).realForward(a)
    got = _full(shape, a.astype(np.float64), _util(shape))
    assert rel_l2(got.ravel(), _want(x).ravel()) <= tol(N, dt)
