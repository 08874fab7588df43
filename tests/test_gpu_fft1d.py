"""GPU parity: 1D FFT ops through the C ABI against the oracle (same inputs as
the reference tests: java.util.Random(20110602), uniform [-1, 1)) and against
the FFTW golden vectors (fft/DoubleFFT_1DTest.java, fft/FloatFFT_1DTest.java).
Tolerance: relative L2 <= 4 * eps * log2(n) of the precision."""
import functools

import numpy as np
import pytest

from tests._helpers import SEED, JavaRandom, rel_l2, rmse, tol

pytestmark = pytest.mark.gpu

# fft/DoubleFFT_1DTest.java:88-90 plus primes on both sides of the Bluestein threshold
SIZES = [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 16, 32, 64, 100, 120, 128, 199, 211, 256, 310, 512, 1024,
         1056, 2048, 8192, 10158, 16384, 32768, 65530, 65536, 131072]
OPS = ["cf", "ci_s", "ci_u", "rf", "rff", "ri_s", "ri_u", "rif_s", "rif_u"]


@functools.lru_cache(maxsize=None)
def _inputs(n):
    return JavaRandom(SEED).uniform_pm1(2 * n)


def _classes():
    import jtransforms_gb300 as J
    return {"f64": (np.float64, J.DoubleFFT_1D), "f32": (np.float32, J.FloatFFT_1D)}


@functools.lru_cache(maxsize=None)
def _plan(prec, n):
    dt, cls = _classes()[prec]
    return cls(n)


def _case(oracle, prec, n, op):
    """Returns (gpu_result, oracle_result) for one op."""
    dt, _ = _classes()[prec]
    f = _plan(prec, n)
    O = oracle
    x = _inputs(n).astype(dt)
    if op in ("cf", "ci_s", "ci_u"):
        a = x.copy()
        b = x.copy()
        if op == "cf":
            f.complexForward(a)
            O.run(O.FFT, O.COMPLEX_FORWARD, [n], b)
        else:
            s = op == "ci_s"
            f.complexInverse(a, s)
            O.run(O.FFT, O.COMPLEX_INVERSE, [n], b, s)
        return a, b
    if op in ("rf", "rff", "rif_s", "rif_u"):
        a = np.zeros(2 * n, dt)
        a[:n] = x[:n]
        b = a.copy()
        if op == "rf":
            f.realForward(a)
            O.run(O.FFT, O.REAL_FORWARD, [n], b)
            return a[:n], b[:n]
        if op == "rff":
            f.realForwardFull(a)
            O.run(O.FFT, O.REAL_FORWARD_FULL, [n], b)
            return a, b
        s = op == "rif_s"
        f.realInverseFull(a, s)
        O.run(O.FFT, O.REAL_INVERSE_FULL, [n], b, s)
        return a, b
    # realInverse of a packed spectrum made by the oracle
    p = x[:n].copy()
    O.run(O.FFT, O.REAL_FORWARD, [n], p)
    a, b = p.copy(), p.copy()
    s = op == "ri_s"
    f.realInverse(a, s)
    O.run(O.FFT, O.REAL_INVERSE, [n], b, s)
    return a, b


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("op", OPS)
@pytest.mark.parametrize("n", SIZES)
def test_fft1d_parity(oracle, prec, op, n):
    a, b = _case(oracle, prec, n, op)
    dt = np.float64 if prec == "f64" else np.float32
    err = rel_l2(a, b)
    assert err <= tol(n, dt), f"n={n} op={op} {prec}: rel L2 {err:.3e} > {tol(n, dt):.3e}"


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_fft1d_golden(golden, prec):
    """testComplexForward on the FFTW files: RMSE < 1e-12 (double), 1e-4 (float)."""
    dt, cls = _classes()[prec]
    for n in golden["sizes"]:
        n = int(n)
        a = golden[f"in{n}"].astype(dt)
        cls(n).complexForward(a)
        assert rmse(a, golden[f"out{n}"]) < (1e-12 if prec == "f64" else 1e-4), n


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("n", [1, 7, 64, 100, 4096, 10158])
def test_offsets_and_bounds(oracle, prec, n):
    import jtransforms_gb300 as J
    dt, cls = _classes()[prec]
    f = cls(n)
    off = 5
    x = _inputs(n).astype(dt)
    buf = np.full(2 * n + off + 3, 7.0, dt)
    buf[off:off + 2 * n] = x
    f.complexForward(buf, off)
    b = x.copy()
    oracle.run(oracle.FFT, oracle.COMPLEX_FORWARD, [n], b)
    assert rel_l2(buf[off:off + 2 * n], b) <= tol(n, dt)
    assert np.all(buf[:off] == 7.0) and np.all(buf[off + 2 * n:] == 7.0)
    with pytest.raises(J.ArrayIndexOutOfBoundsException):
        f.complexForward(np.zeros(2 * n - 1, dt))
    with pytest.raises(J.ArrayIndexOutOfBoundsException):
        f.realForward(np.zeros(n, dt), 1)
    with pytest.raises(TypeError):
        f.complexForward(np.zeros(2 * n, np.float32 if dt == np.float64 else np.float64))


@pytest.mark.parametrize("prec,n,batch,gap,op", [("f32", 1024, 50000, 0, "cf"), ("f32", 1024, 20001, 6, "cf"),
                                                ("f64", 4096, 5000, 2, "ci"), ("f32", 1 << 20, 40, 0, "rf"),
                                                ("f64", 1000, 3, 4, "cf")])
def test_host_batch_pieces(prec, n, batch, gap, op):
    """jt_execute_batch on a host array of many pieces (copy in, transform and
    copy out overlapped through a ring of device buffers), with and without a
    gap between arrays and an offset: identical to the device-array path."""
    import torch
    from jtransforms_gb300 import _native as N
    dt = np.float64 if prec == "f64" else np.float32
    cls = _classes()[prec][1]
    f = cls(n)
    ext = n if op == "rf" else 2 * n
    dist = ext + gap
    off = 3
    code = {"cf": N.COMPLEX_FORWARD, "ci": N.COMPLEX_INVERSE, "rf": N.REAL_FORWARD}[op]
    rng = np.random.default_rng(n + batch)
    host = rng.uniform(-1, 1, off + dist * batch).astype(dt)
    keep = host.copy()
    f.plan.execute(code, host, off, op == "ci", batch=batch, dist=dist)
    dense = np.stack([keep[off + b * dist: off + b * dist + ext] for b in range(batch)])
    dev = torch.from_numpy(dense.ravel().copy()).cuda()
    f.plan.execute(code, dev, 0, op == "ci", batch=batch, dist=ext)
    got = np.stack([host[off + b * dist: off + b * dist + ext] for b in range(batch)])
    assert np.array_equal(got, dev.cpu().numpy().reshape(batch, ext))
    # the gaps and the prefix are untouched
    assert np.array_equal(host[:off], keep[:off])
    for b in range(min(batch, 50)):
        s = off + b * dist + ext
        assert np.array_equal(host[s:s + gap], keep[s:s + gap])


@pytest.mark.parametrize("n", [4096, 1000, 4099])
def test_round_trips(n):
    """complexForward then complexInverse(scale) and realForward then
    realInverse(scale) return the input (fft/DoubleFFT_1DTest.java:210-300)."""
    import jtransforms_gb300 as J
    x = _inputs(n)
    f = J.DoubleFFT_1D(n)
    a = x.copy()
    f.complexForward(a)
    f.complexInverse(a, True)
    assert rmse(a, x) < 1e-12
    r = x[:n].copy()
    f.realForward(r)
    f.realInverse(r, True)
    assert rmse(r, x[:n]) < 1e-12


@pytest.mark.parametrize("prec,n", [("f32", 8192), ("f32", 16384), ("f64", 4096), ("f64", 8192)])
@pytest.mark.parametrize("gap", [0, 8, 2])
def test_long_lines_batched_with_gaps(prec, n, gap):
    """The one-pass kernels of the longest lines (the two-stage pipeline at
    float 8192 and double 4096, the prefix-prefetch kernel at float 16384
    and double 8192) over a device batch whose arrays sit `gap` elements
    apart: 0 and 8 keep TMA's 16-byte rules (contiguous lines, strided
    lines); 2 floats break them (the plain kernel); against an FP64 FFT."""
    import torch
    from jtransforms_gb300 import _native as N
    if prec == "f64" and gap == 2:
        pytest.skip("a double complex line is 16-byte aligned at every even gap")
    dt, _ = _classes()[prec]
    f = _plan(prec, n)
    batch, ext = 5, 2 * n
    dist = ext + gap
    rng = np.random.default_rng(n + gap)
    host = rng.uniform(-1, 1, dist * batch).astype(dt)
    dev = torch.from_numpy(host.copy()).cuda()
    f.plan.execute(N.COMPLEX_FORWARD, dev, 0, False, batch=batch, dist=dist)
    got = dev.cpu().numpy()
    for b in range(batch):
        z = host[b * dist:b * dist + ext].astype(np.float64)
        y = np.fft.fft(z[0::2] + 1j * z[1::2])
        want = np.empty(ext)
        want[0::2], want[1::2] = y.real, y.imag
        assert rel_l2(got[b * dist:b * dist + ext], want) <= tol(n, dt)
        assert np.array_equal(got[b * dist + ext:(b + 1) * dist], host[b * dist + ext:(b + 1) * dist])
