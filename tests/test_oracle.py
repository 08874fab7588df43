"""CPU tests: the oracle against JTransforms' golden vectors and the identities
its tests rely on (fft/DoubleFFT_1DTest.java, dct/DoubleDCT_1DTest.java ...)."""
import os

import numpy as np
import pytest
import scipy.fft as sf

from tests._helpers import SEED, JavaRandom, rel_l2, rmse

# JTransforms checkout whose test resources hold the five larger golden files
# (JTRANSFORMS_REFERENCE; the test skips when it is unset or absent)
REF_RES = os.path.join(os.environ.get("JTRANSFORMS_REFERENCE", ""), "src", "test", "resources")


def test_java_random_matches_spec():
    # first values of new Random(42).nextDouble() from the Java SE LCG definition
    r = JavaRandom(42)
    v = [r.nextDouble() for _ in range(3)]
    assert abs(v[0] - 0.7275636800328681) < 1e-16
    assert abs(v[1] - 0.6832234717598454) < 1e-16
    assert abs(v[2] - 0.30871945533265976) < 1e-16


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_oracle_golden_complex_forward(oracle, golden, prec):
    """testComplexForward: RMSE < 1e-12 (double) / 1e-4 (float cast of the same
    files), fft/DoubleFFT_1DTest.java:196-206, fft/FloatFFT_1DTest.java:202-218."""
    for n in golden["sizes"]:
        x, y = golden[f"in{n}"], golden[f"out{n}"]
        a = x.copy() if prec == "f64" else x.astype(np.float32)
        oracle.run(oracle.FFT, oracle.COMPLEX_FORWARD, [int(n)], a)
        assert rmse(a, y) < (1e-12 if prec == "f64" else 1e-4), n


@pytest.mark.skipif(not os.environ.get("JTRANSFORMS_REFERENCE") or not os.path.isdir(REF_RES),
                    reason="reference test resources not present (set JTRANSFORMS_REFERENCE)")
def test_oracle_golden_large():
    from oracle import oracle as O
    for n in (16384, 32768, 65530, 65536, 131072):
        x = np.fromfile(os.path.join(REF_RES, f"fftw{n}.in"), "<f8")
        y = np.fromfile(os.path.join(REF_RES, f"fftw{n}.out"), "<f8")
        O.run(O.FFT, O.COMPLEX_FORWARD, [n], x)
        assert rmse(x, y) < 1e-12


def test_plan_choice(oracle):
    # fft/DoubleFFT_1D.java:117-188 with getReminder(n, {4,2,3,5})
    assert oracle.plan_kind(4096) == oracle.SPLIT_RADIX
    assert oracle.plan_kind(310) == oracle.MIXED_RADIX
    assert oracle.plan_kind(10158) == oracle.BLUESTEIN
    assert oracle.plan_kind(65530) == oracle.BLUESTEIN
    assert oracle.plan_kind(199) == oracle.MIXED_RADIX  # prime < 211
    assert oracle.plan_kind(211) == oracle.BLUESTEIN
    assert oracle.bluestein_size(10158) == 32768


def _pack(F, n):
    a = np.zeros(n)
    a[0] = F[0].real
    if n % 2 == 0:
        if n > 1:
            a[1] = F[n // 2].real
        for k in range(1, n // 2):
            a[2 * k], a[2 * k + 1] = F[k].real, F[k].imag
    else:
        h = (n - 1) // 2
        if n > 1:
            a[1] = F[h].imag
        for k in range(1, h):
            a[2 * k], a[2 * k + 1] = F[k].real, F[k].imag
        if h >= 1:
            a[2 * h] = F[h].real
    return a


SIZES_1D = [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 16, 17, 32, 64, 100, 120, 128, 199, 211, 256, 310, 512,
            1024, 1056, 2048, 4096, 10158]


@pytest.mark.parametrize("n", SIZES_1D)
def test_oracle_1d_semantics(oracle, n):
    O = oracle
    rnd = JavaRandom(SEED)
    x = rnd.uniform_pm1(n)
    F = np.fft.fft(x)
    a = np.zeros(2 * n); a[:n] = x
    O.run(O.FFT, O.REAL_FORWARD, [n], a)
    assert rel_l2(a[:n], _pack(F, n)) < 1e-14
    b = np.zeros(2 * n); b[:n] = x
    O.run(O.FFT, O.REAL_FORWARD_FULL, [n], b)
    assert rel_l2(b[0::2] + 1j * b[1::2], F) < 1e-14
    # realInverse: unscaled gives n/2 * x for power-of-two n > 1, n * x otherwise
    c = a[:n].copy(); O.run(O.FFT, O.REAL_INVERSE, [n], c, False)
    fac = n / 2 if (n & (n - 1)) == 0 and n > 1 else n
    assert rel_l2(c / fac, x) < 1e-14
    c = a[:n].copy(); O.run(O.FFT, O.REAL_INVERSE, [n], c, True)
    assert rel_l2(c, x) < 1e-14
    g = np.zeros(2 * n); g[:n] = x
    O.run(O.FFT, O.REAL_INVERSE_FULL, [n], g, True)
    assert rel_l2(g[0::2] + 1j * g[1::2], np.fft.ifft(x)) < 1e-14
    # DCT / DST orthonormal, DHT = Re F - Im F
    y = x.copy(); O.run(O.DCT, O.FORWARD, [n], y, True)
    assert rel_l2(y, sf.dct(x, 2, norm="ortho")) < 1e-14
    y = x.copy(); O.run(O.DCT, O.INVERSE, [n], y, True)
    assert rel_l2(y, sf.idct(x, 2, norm="ortho")) < 1e-14
    if n > 1:
        y = x.copy(); O.run(O.DST, O.FORWARD, [n], y, True)
        assert rel_l2(y, sf.dst(x, 2, norm="ortho")) < 1e-14
        # unscaled DCT-II: no factor 2 on power-of-two sizes, factor 2 otherwise
        y = x.copy(); O.run(O.DCT, O.FORWARD, [n], y, False)
        f2 = 1 if (n & (n - 1)) == 0 else 2
        assert rel_l2(y, f2 * sf.dct(x, 2) / 2) < 1e-14
    y = x.copy(); O.run(O.DHT, O.FORWARD, [n], y)
    assert rel_l2(y, F.real - F.imag) < 1e-14


def _unpack2d(a, rows, cols):
    """Full spectrum from the packed 2D layout documented at
    fft/DoubleFFT_2D.java:788-815."""
    A = a.reshape(rows, cols)
    F = np.full((rows, cols), np.nan + 0j)
    for k1 in range(rows):
        for k2 in range(1, cols // 2):
            F[k1, k2] = A[k1, 2 * k2] + 1j * A[k1, 2 * k2 + 1]
    for k1 in range(1, rows // 2):
        F[k1, 0] = A[k1, 0] + 1j * A[k1, 1]
        F[k1, cols // 2] = A[rows - k1, 1] - 1j * A[rows - k1, 0]
    F[0, 0] = A[0, 0]
    F[0, cols // 2] = A[0, 1]
    F[rows // 2, 0] = A[rows // 2, 0]
    F[rows // 2, cols // 2] = A[rows // 2, 1]
    for k1 in range(rows):
        for k2 in range(cols):
            if np.isnan(F[k1, k2]):
                F[k1, k2] = np.conj(F[(-k1) % rows, (-k2) % cols])
    return F


@pytest.mark.parametrize("shape", [(2, 2), (4, 8), (16, 16), (32, 64)])
def test_oracle_2d_real_packed(oracle, shape):
    rows, cols = shape
    x = np.random.default_rng(1).uniform(-1, 1, shape)
    a = x.ravel().copy()
    oracle.run(oracle.FFT, oracle.REAL_FORWARD, list(shape), a)
    assert rel_l2(_unpack2d(a, rows, cols), np.fft.fft2(x)) < 1e-14
    oracle.run(oracle.FFT, oracle.REAL_INVERSE, list(shape), a, True)
    assert rel_l2(a, x.ravel()) < 1e-14


def fill_symmetric_3d(a, slices, rows, cols):
    """Expands the packed 3D realForward result (first slices*rows*cols
    values of `a`, length 2*slices*rows*cols) into the full interleaved
    spectrum, as the reference test does (fft/DoubleFFT_3DTest.java:431-558)."""
    twon3, n2d2, n1d2 = 2 * cols, rows // 2, slices // 2
    ss, rs = rows * cols, cols
    tss, trs = rows * twon3, twon3
    for s in range(slices - 1, 0, -1):
        for r in range(rows):
            for c in range(0, cols, 2):
                i1, i2 = s * ss + r * rs + c, 2 * s * ss + 2 * r * rs + c
                a[i2], a[i1] = a[i1], 0
                a[i2 + 1], a[i1 + 1] = a[i1 + 1], 0
    for r in range(1, rows):
        for c in range(0, cols, 2):
            i1, i2 = (rows - r) * rs + c, (rows - r) * trs + c
            a[i2], a[i1] = a[i1], 0
            a[i2 + 1], a[i1 + 1] = a[i1 + 1], 0
    for s in range(slices):
        i3, i5 = ((slices - s) % slices) * tss, s * tss
        for r in range(rows):
            i4, i6 = ((rows - r) % rows) * trs, r * trs
            for c in range(1, cols, 2):
                i1, i2 = i3 + i4 + twon3 - c, i5 + i6 + c
                a[i1] = -a[i2 + 2]
                a[i1 - 1] = a[i2 + 1]
    for s in range(slices):
        i5, i6 = ((slices - s) % slices) * tss, s * tss
        for r in range(1, n2d2):
            i4 = i6 + (rows - r) * trs
            i1, i2, i3 = i5 + r * trs + cols, i4 + cols, i4 + 1
            a[i1] = a[i3]
            a[i2] = a[i3]
            a[i1 + 1] = -a[i4]
            a[i2 + 1] = a[i4]
    for s in range(slices):
        i3, i4 = ((slices - s) % slices) * tss, s * tss
        for r in range(1, n2d2):
            i1, i2 = i3 + (rows - r) * trs, i4 + r * trs
            a[i1] = a[i2]
            a[i1 + 1] = -a[i2 + 1]
    for s in range(1, n1d2):
        i1, i2, i3 = s * tss, (slices - s) * tss, n2d2 * trs
        i4, i5 = i1 + i3, i2 + i3
        a[i1 + cols] = a[i2 + 1]
        a[i2 + cols] = a[i2 + 1]
        a[i1 + cols + 1] = -a[i2]
        a[i2 + cols + 1] = a[i2]
        a[i4 + cols] = a[i5 + 1]
        a[i5 + cols] = a[i5 + 1]
        a[i4 + cols + 1] = -a[i5]
        a[i5 + cols + 1] = a[i5]
        a[i2] = a[i1]
        a[i2 + 1] = -a[i1 + 1]
        a[i5] = a[i4]
        a[i5 + 1] = -a[i4 + 1]
    a[cols] = a[1]
    a[1] = 0
    i1, i2 = n2d2 * trs, n1d2 * tss
    i3 = i1 + i2
    a[i1 + cols] = a[i1 + 1]
    a[i1 + 1] = 0
    a[i2 + cols] = a[i2 + 1]
    a[i2 + 1] = 0
    a[i3 + cols] = a[i3 + 1]
    a[i3 + 1] = 0
    a[i2 + cols + 1] = 0
    a[i3 + cols + 1] = 0
    return a


@pytest.mark.parametrize("shape", [(2, 2, 2), (4, 8, 16), (8, 4, 2), (16, 16, 16), (4, 32, 8)])
def test_oracle_3d_real_packed(oracle, shape):
    """Pinned like the reference test (fft/DoubleFFT_3DTest.java:565-592):
    the packed result, expanded by fillSymmetric, equals the full complex
    forward transform; realInverse(scale) restores the input."""
    s_, r_, c_ = shape
    N = s_ * r_ * c_
    x = np.random.default_rng(3).uniform(0, 1, shape)
    a = np.zeros(2 * N)
    a[:N] = x.ravel()
    oracle.run(oracle.FFT, oracle.REAL_FORWARD, list(shape), a[:N])
    packed = a[:N].copy()
    full = fill_symmetric_3d(a, s_, r_, c_)
    F = np.fft.fftn(x)
    want = np.empty(2 * N)
    want[0::2] = F.real.ravel()
    want[1::2] = F.imag.ravel()
    assert rel_l2(full, want) < 1e-14
    oracle.run(oracle.FFT, oracle.REAL_INVERSE, list(shape), packed, True)
    assert rel_l2(packed, x.ravel()) < 1e-14


@pytest.mark.parametrize("dims", [(3, 5), (6, 10), (5, 7, 3), (4, 4, 4), (8, 6, 10)])
def test_oracle_nd(oracle, dims):
    O = oracle
    rng = np.random.default_rng(2)
    z = rng.standard_normal(2 * int(np.prod(dims)))
    a = z.copy(); O.run(O.FFT, O.COMPLEX_FORWARD, list(dims), a)
    assert rel_l2(a[0::2] + 1j * a[1::2], np.fft.fftn((z[0::2] + 1j * z[1::2]).reshape(dims)).ravel()) < 1e-14
    x = rng.uniform(-1, 1, dims)
    y = x.ravel().copy(); O.run(O.DCT, O.FORWARD, list(dims), y, True)
    assert rel_l2(y, sf.dctn(x, 2, norm="ortho").ravel()) < 1e-14
    y = x.ravel().copy(); O.run(O.DST, O.FORWARD, list(dims), y, True)
    assert rel_l2(y, sf.dstn(x, 2, norm="ortho").ravel()) < 1e-14
    Fx = np.fft.fftn(x)
    y = x.ravel().copy(); O.run(O.DHT, O.FORWARD, list(dims), y)
    assert rel_l2(y, (Fx.real - Fx.imag).ravel()) < 1e-14  # cas of the summed phase
    O.run(O.DHT, O.INVERSE, list(dims), y, True)
    assert rel_l2(y, x.ravel()) < 1e-14
