"""GPU parity: 2D/3D FFT and DCT/DST/DHT (1D/2D/3D) through the C ABI against
the oracle (fft/DoubleFFT_2DTest.java, fft/DoubleFFT_3DTest.java,
dct/DoubleDCT_*Test.java, dst/..., dht/...)."""
import numpy as np
import pytest

from tests._helpers import SEED, JavaRandom, rel_l2, rmse, tol

pytestmark = pytest.mark.gpu


def _x(count, seed=SEED):
    rng = np.random.default_rng(seed)
    return rng.uniform(-1, 1, count)


SHAPES_2D = [(2, 2), (3, 5), (4, 8), (16, 16), (13, 7), (100, 120), (128, 256), (310, 64), (511, 512), (1024, 1024)]
SHAPES_3D = [(2, 2, 2), (3, 5, 7), (4, 8, 16), (16, 16, 16), (10, 12, 9), (64, 32, 128), (128, 128, 128)]


def _fft_cls(nd, prec):
    import jtransforms_gb300 as J
    return {(2, "f64"): J.DoubleFFT_2D, (2, "f32"): J.FloatFFT_2D, (3, "f64"): J.DoubleFFT_3D, (3, "f32"): J.FloatFFT_3D}[(nd, prec)]


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("shape", SHAPES_2D + SHAPES_3D)
def test_fft_nd_complex(oracle, prec, shape):
    dt = np.float64 if prec == "f64" else np.float32
    N = int(np.prod(shape))
    f = _fft_cls(len(shape), prec)(*shape)
    x = _x(2 * N).astype(dt)
    a, b = x.copy(), x.copy()
    f.complexForward(a)
    oracle.run(oracle.FFT, oracle.COMPLEX_FORWARD, list(shape), b)
    assert rel_l2(a, b) <= tol(N, dt)
    f.complexInverse(a, True)
    oracle.run(oracle.FFT, oracle.COMPLEX_INVERSE, list(shape), b, True)
    assert rel_l2(a, b) <= tol(N, dt)
    assert rel_l2(a, x) <= 2 * tol(N, dt)


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("shape", SHAPES_2D + SHAPES_3D)
def test_fft_nd_real_full(oracle, prec, shape):
    dt = np.float64 if prec == "f64" else np.float32
    N = int(np.prod(shape))
    f = _fft_cls(len(shape), prec)(*shape)
    a = np.zeros(2 * N, dt)
    a[:N] = _x(N)
    b = a.copy()
    f.realForwardFull(a)
    oracle.run(oracle.FFT, oracle.REAL_FORWARD_FULL, list(shape), b)
    assert rel_l2(a, b) <= tol(N, dt)
    a[:] = 0
    a[:N] = _x(N, 7)
    b = a.copy()
    f.realInverseFull(a, True)
    oracle.run(oracle.FFT, oracle.REAL_INVERSE_FULL, list(shape), b, True)
    assert rel_l2(a, b) <= tol(N, dt)


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("shape", [(2, 2), (2, 8), (4, 4), (16, 8), (64, 128), (256, 256), (2048, 2048)])
def test_fft_2d_real_packed(oracle, prec, shape):
    dt = np.float64 if prec == "f64" else np.float32
    N = int(np.prod(shape))
    f = _fft_cls(2, prec)(*shape)
    x = _x(N).astype(dt)
    a, b = x.copy(), x.copy()
    f.realForward(a)
    oracle.run(oracle.FFT, oracle.REAL_FORWARD, list(shape), b)
    assert rel_l2(a, b) <= tol(N, dt)
    for s in (True, False):
        c, d = a.copy(), b.copy()
        f.realInverse(c, s)
        oracle.run(oracle.FFT, oracle.REAL_INVERSE, list(shape), d, s)
        assert rel_l2(c, d) <= tol(N, dt)


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("shape", [(2, 2, 2), (2, 4, 8), (4, 8, 16), (8, 4, 2), (16, 16, 16), (32, 64, 16),
                                   (128, 128, 128)])
def test_fft_3d_real_packed(oracle, prec, shape):
    """fft/DoubleFFT_3D.java realForward / realInverse packed layout
    (fft/DoubleFFT_3DTest.java:565-592, :868-895)."""
    dt = np.float64 if prec == "f64" else np.float32
    N = int(np.prod(shape))
    f = _fft_cls(3, prec)(*shape)
    x = _x(N).astype(dt)
    a, b = x.copy(), x.copy()
    f.realForward(a)
    oracle.run(oracle.FFT, oracle.REAL_FORWARD, list(shape), b)
    assert rel_l2(a, b) <= tol(N, dt)
    for s in (True, False):
        c, d = a.copy(), b.copy()
        f.realInverse(c, s)
        oracle.run(oracle.FFT, oracle.REAL_INVERSE, list(shape), d, s)
        assert rel_l2(c, d) <= tol(N, dt)
    c = a.copy()
    f.realInverse(c, True)
    assert rel_l2(c, x) <= 2 * tol(N, dt)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_jagged_rows(prec):
    """double[][] / double[][][] overloads (fft/DoubleFFT_2D.java:345,
    fft/DoubleFFT_3D.java:542, dct/DoubleDCT_2D.java:104): lists of row
    arrays give the flat array's results, realForwardFull reads the first
    half of each 2*columns row (fft/DoubleFFT_2D.java:1010-1021)."""
    import jtransforms_gb300 as J
    dt = np.float64 if prec == "f64" else np.float32
    rows, cols = 8, 16
    f = _fft_cls(2, prec)(rows, cols)
    x = _x(2 * rows * cols).astype(dt)
    flat = x.copy()
    f.complexForward(flat)
    jag = [x[r * 2 * cols:(r + 1) * 2 * cols].copy() for r in range(rows)]
    f.complexForward(jag)
    assert np.array_equal(np.concatenate(jag), flat)
    # packed real, rows of `cols`
    xr = x[: rows * cols].copy()
    flat = xr.copy()
    f.realForward(flat)
    jag = [xr[r * cols:(r + 1) * cols].copy() for r in range(rows)]
    f.realForward(jag)
    assert np.array_equal(np.concatenate(jag), flat)
    # full real: input in the first half of each 2*cols row
    flat = np.zeros(2 * rows * cols, dt)
    flat[: rows * cols] = xr
    f.realForwardFull(flat)
    jag = [np.concatenate([xr[r * cols:(r + 1) * cols], np.zeros(cols, dt)]) for r in range(rows)]
    f.realForwardFull(jag)
    assert np.array_equal(np.concatenate(jag), flat)
    # 3D nested lists and a 2D DCT of rows
    g = _fft_cls(3, prec)(4, 2, 8)
    y = _x(2 * 64).astype(dt)
    flat = y.copy()
    g.complexForward(flat)
    nest = [[y[(s * 2 + r) * 16:(s * 2 + r + 1) * 16].copy() for r in range(2)] for s in range(4)]
    g.complexForward(nest)
    assert np.array_equal(np.concatenate([row for sl in nest for row in sl]), flat)
    d = getattr(J, ("Double" if prec == "f64" else "Float") + "DCT_2D")(rows, cols)
    flat = xr.copy()
    d.forward(flat, True)
    jag = [xr[r * cols:(r + 1) * cols].copy() for r in range(rows)]
    d.forward(jag, True)
    assert np.array_equal(np.concatenate(jag), flat)
    with pytest.raises(TypeError):
        f.complexForward([np.zeros(2 * cols, np.float32 if dt == np.float64 else np.float64)] * rows)
    with pytest.raises(J.IllegalArgumentException):
        f.complexForward(jag, 2)


def test_fft_3d_real_requires_pow2():
    import jtransforms_gb300 as J
    f = J.DoubleFFT_3D(4, 6, 8)
    with pytest.raises(J.IllegalArgumentException):
        f.realForward(np.zeros(192))


def test_fft_2d_real_requires_pow2():
    import jtransforms_gb300 as J
    f = J.DoubleFFT_2D(6, 8)
    with pytest.raises(J.IllegalArgumentException):
        f.realForward(np.zeros(48))


def _r2r_cls(kind, nd, prec):
    import jtransforms_gb300 as J
    p = "Double" if prec == "f64" else "Float"
    return getattr(J, f"{p}{kind}_{nd}D")


R2R_1D = [1, 2, 3, 4, 5, 8, 16, 17, 31, 64, 100, 120, 128, 211, 256, 310, 512, 1000, 1024, 4096, 10158, 16384, 65536]


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("kind", ["DCT", "DST", "DHT"])
@pytest.mark.parametrize("n", R2R_1D)
def test_r2r_1d(oracle, prec, kind, n):
    dt = np.float64 if prec == "f64" else np.float32
    code = {"DCT": oracle.DCT, "DST": oracle.DST, "DHT": oracle.DHT}[kind]
    f = _r2r_cls(kind, 1, prec)(n)
    x = JavaRandom(SEED).uniform_pm1(n).astype(dt)
    for s in (True, False):
        a, b = x.copy(), x.copy()
        if kind == "DHT":
            f.forward(a)
            oracle.run(code, oracle.FORWARD, [n], b)
        else:
            f.forward(a, s)
            oracle.run(code, oracle.FORWARD, [n], b, s)
        assert rel_l2(a, b) <= tol(n, dt), (kind, n, s, "forward")
        c, d = x.copy(), x.copy()
        f.inverse(c, s)
        oracle.run(code, oracle.INVERSE, [n], d, s)
        assert rel_l2(c, d) <= tol(n, dt), (kind, n, s, "inverse")
    # testScaled round trip (dct/DoubleDCT_1DTest.java)
    a = x.copy()
    if kind == "DHT":
        f.forward(a)
    else:
        f.forward(a, True)
    f.inverse(a, True)
    assert rmse(a, x) < (1e-12 if prec == "f64" else 1e-5)


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("kind", ["DCT", "DST", "DHT"])
@pytest.mark.parametrize("shape", [(2, 2), (4, 6), (16, 16), (100, 120), (1024, 1024), (2, 3, 4), (16, 16, 16), (10, 12, 14), (128, 128, 128)])
def test_r2r_nd(oracle, prec, kind, shape):
    dt = np.float64 if prec == "f64" else np.float32
    code = {"DCT": oracle.DCT, "DST": oracle.DST, "DHT": oracle.DHT}[kind]
    N = int(np.prod(shape))
    f = _r2r_cls(kind, len(shape), prec)(*shape)
    x = _x(N, 11).astype(dt)
    for s in (True, False):
        a, b = x.copy(), x.copy()
        if kind == "DHT":
            f.forward(a)
            oracle.run(code, oracle.FORWARD, list(shape), b)
        else:
            f.forward(a, s)
            oracle.run(code, oracle.FORWARD, list(shape), b, s)
        assert rel_l2(a, b) <= tol(N, dt), (kind, shape, s)
        c, d = x.copy(), x.copy()
        f.inverse(c, s)
        oracle.run(code, oracle.INVERSE, list(shape), d, s)
        assert rel_l2(c, d) <= tol(N, dt), (kind, shape, s, "inverse")
