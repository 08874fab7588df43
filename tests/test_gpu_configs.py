"""GPU parity on the benchmark workloads themselves, through the C ABI:

* DoubleFFT_1D(4096): complexForward then complexInverse(scale=true) on 256
  independent arrays in one batched call, on a host array and on a device
  tensor, against the oracle (fft/DoubleFFT_1DTest.java testComplexForward /
  testComplexInverseScaled, batched as the benchmark loops them).
* DoubleFFT_3D(256, 256, 256).complexForward on N(0,1) complex128, against the
  oracle's row-column composition (fft/DoubleFFT_3DTest.java), plus the
  scaled inverse round trip.
* FloatFFT_1D at 2^10, 2^14, 2^18, 2^20 and 2^24 with the pass splits the
  compiled plan table picks (one pass, 1024 x 256, 1024 x 1024, three
  passes), batched, forward and scaled inverse, on input set (a) N(0,1) and
  set (b) 60 dB (8 unit complex exponentials at random bins plus
  1e-3 N(0,1)): against an FP64 FFT, and side by side against the oracle's
  FloatFFT restatement with its float-angle twiddles
  (fft/FloatFFT_1D.java:1484-1507).

Tolerance: relative L2 <= 4 * eps * log2(N) of the working precision
(the same bound as every parity test here); against the float oracle the
budget is the GPU's and the oracle's together (2x)."""
import numpy as np
import pytest

from tests._helpers import rel_l2, tol

pytestmark = pytest.mark.gpu

SEED = 20110602


def _fp64_fft(x, n, inverse=False, scale=False):
    z = x.astype(np.float64).reshape(-1, n, 2)
    c = z[..., 0] + 1j * z[..., 1]
    y = (np.fft.ifft(c, axis=1) * (1 if scale else n)) if inverse else np.fft.fft(c, axis=1)
    out = np.empty(x.size)
    out[0::2] = y.real.ravel()
    out[1::2] = y.imag.ravel()
    return out


def _sixty_db(n, batch, rng):
    """Set (b): 8 unit-amplitude complex exponentials at random bins plus
    1e-3 N(0,1), per transform."""
    t = np.arange(n)
    out = np.empty((batch, n), np.complex128)
    for b in range(batch):
        bins = rng.integers(0, n, 8)
        ph = rng.uniform(0, 2 * np.pi, 8)
        z = np.zeros(n, np.complex128)
        for k, p in zip(bins, ph):
            z += np.exp(1j * (2 * np.pi * ((t * int(k)) % n) / n + p))
        out[b] = z + 1e-3 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    x = np.empty(2 * n * batch)
    x[0::2] = out.real.ravel()
    x[1::2] = out.imag.ravel()
    return x


@pytest.mark.parametrize("where", ["host", "device"])
def test_double_4096_x256_forward_then_scaled_inverse(oracle, where):
    import torch

    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    n, batch = 4096, 256
    x = np.random.default_rng(SEED).uniform(-1, 1, 2 * n * batch)
    f = J.DoubleFFT_1D(n)
    want = x.copy()
    oracle.run_batch(oracle.FFT, oracle.COMPLEX_FORWARD, [n], want, batch, 2 * n)
    if where == "host":
        a = x.copy()
        f.plan.execute(N.COMPLEX_FORWARD, a, 0, False, batch=batch, dist=2 * n)
    else:
        d = torch.from_numpy(x.copy()).cuda()
        f.plan.execute(N.COMPLEX_FORWARD, d, 0, False, batch=batch, dist=2 * n)
        torch.cuda.synchronize()
        a = d.cpu().numpy()
    for b in (0, 1, batch // 2, batch - 1):
        s = slice(2 * n * b, 2 * n * (b + 1))
        assert rel_l2(a[s], want[s]) <= tol(n, np.float64), b
    assert rel_l2(a, want) <= tol(n, np.float64)
    oracle.run_batch(oracle.FFT, oracle.COMPLEX_INVERSE, [n], want, batch, 2 * n, True)
    if where == "host":
        f.plan.execute(N.COMPLEX_INVERSE, a, 0, True, batch=batch, dist=2 * n)
    else:
        f.plan.execute(N.COMPLEX_INVERSE, d, 0, True, batch=batch, dist=2 * n)
        torch.cuda.synchronize()
        a = d.cpu().numpy()
    assert rel_l2(a, want) <= tol(n, np.float64)
    assert rel_l2(a, x) <= 2 * tol(n, np.float64)


def test_double_3d_256_cubed(oracle):
    import jtransforms_gb300 as J
    shape = (256, 256, 256)
    N = 256 ** 3
    rng = np.random.default_rng(SEED)
    x = rng.standard_normal(2 * N)
    f = J.DoubleFFT_3D(*shape)
    a, b = x.copy(), x.copy()
    f.complexForward(a)
    oracle.run(oracle.FFT, oracle.COMPLEX_FORWARD, list(shape), b)
    assert rel_l2(a, b) <= tol(N, np.float64)
    # one pencil along each axis against numpy's FP64 transform of the cube
    z = (x[0::2] + 1j * x[1::2]).reshape(shape)
    ref = np.fft.fftn(z)
    got = (a[0::2] + 1j * a[1::2]).reshape(shape)
    for idx in ((slice(None), 3, 7), (5, slice(None), 200), (255, 128, slice(None))):
        assert rel_l2(got[idx], ref[idx]) <= tol(N, np.float64)
    f.complexInverse(a, True)
    assert rel_l2(a, x) <= 2 * tol(N, np.float64)


# (log2 n, batch, expected algorithm from the plan table: 0 one pass,
# 1 two passes, 4 three passes)
CONFIG4 = [(10, 64, 0), (14, 8, 0), (18, 4, 1), (20, 2, 1), (24, 1, 4)]


@pytest.mark.parametrize("inputs", ["a", "b"])
@pytest.mark.parametrize("lg,batch,algo", CONFIG4)
def test_float_config4_table_splits(oracle, lg, batch, algo, inputs):
    import torch

    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    n = 1 << lg
    rng = np.random.default_rng(SEED + lg)
    x64 = rng.standard_normal(2 * n * batch) if inputs == "a" else _sixty_db(n, batch, rng)
    x = x64.astype(np.float32)
    f = J.FloatFFT_1D(n)
    assert f.plan.algorithm(0) == algo
    d = torch.from_numpy(x.copy()).cuda()
    f.plan.execute(N.COMPLEX_FORWARD, d, 0, False, batch=batch, dist=2 * n)
    torch.cuda.synchronize()
    got = d.cpu().numpy()
    want64 = _fp64_fft(x, n)
    assert rel_l2(got, want64) <= tol(n, np.float32)
    # the oracle's FloatFFT restatement (float-angle twiddles), side by side
    fo = x.copy()
    oracle.run_batch(oracle.FFT, oracle.COMPLEX_FORWARD, [n], fo, batch, 2 * n)
    assert rel_l2(fo, want64) <= tol(n, np.float32)
    assert rel_l2(got, fo) <= 2 * tol(n, np.float32)
    # scaled inverse brings the spectrum back
    f.plan.execute(N.COMPLEX_INVERSE, d, 0, True, batch=batch, dist=2 * n)
    torch.cuda.synchronize()
    back = d.cpu().numpy()
    assert rel_l2(back, x) <= 2 * tol(n, np.float32)
    # and the scaled inverse alone matches FP64 on the same input
    e = torch.from_numpy(x.copy()).cuda()
    f.plan.execute(N.COMPLEX_INVERSE, e, 0, True, batch=batch, dist=2 * n)
    torch.cuda.synchronize()
    assert rel_l2(e.cpu().numpy(), _fp64_fft(x, n, inverse=True, scale=True)) <= tol(n, np.float32)
