"""GPU parity of the large Float lengths (three passes from 2^21 up, two
passes below): complexForward / complexInverse against an FP64 FFT of the
same input and against the two-pass plan, and realForward of a length whose
half-length complex FFT takes three passes.  Tolerance: relative L2 <=
4 * eps_float * log2(n) (the benchmark spec bound, against FP64)."""
import numpy as np
import pytest

from tests._helpers import rel_l2, tol

pytestmark = pytest.mark.gpu


def _fp64_fft(x, n, inverse=False, scale=False):
    z = x.astype(np.float64).reshape(-1, n, 2)
    c = z[..., 0] + 1j * z[..., 1]
    y = (np.fft.ifft(c, axis=1) * (1 if scale else n)) if inverse else np.fft.fft(c, axis=1)
    out = np.empty(x.size)
    out[0::2] = y.real.ravel()
    out[1::2] = y.imag.ravel()
    return out


@pytest.mark.parametrize("lg,batch", [(21, 2), (22, 1), (23, 1), (24, 1)])
def test_three_pass_complex(lg, batch):
    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    n = 1 << lg
    f = J.FloatFFT_1D(n)
    assert f.plan.algorithm(0) == 4  # three passes
    x = np.random.default_rng(lg).standard_normal(2 * n * batch).astype(np.float32)
    a = x.copy()
    f.plan.execute(N.COMPLEX_FORWARD, a, 0, False, batch=batch, dist=2 * n)
    assert rel_l2(a, _fp64_fft(x, n)) <= tol(n, np.float32)
    for s in (True, False):
        c = x.copy()
        f.plan.execute(N.COMPLEX_INVERSE, c, 0, s, batch=batch, dist=2 * n)
        assert rel_l2(c, _fp64_fft(x, n, inverse=True, scale=s)) <= tol(n, np.float32)


def test_three_pass_matches_two_pass():
    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    n = 1 << 22
    x = np.random.default_rng(5).standard_normal(2 * n).astype(np.float32)
    a = x.copy()
    J.FloatFFT_1D(n).complexForward(a)
    prev = N.set_option(N.OPT_THREEPASS_MIN_LOG2, 0)
    try:
        g = J.FloatFFT_1D(n)
        assert g.plan.algorithm(0) == 1  # two passes
        b = x.copy()
        g.complexForward(b)
    finally:
        N.set_option(N.OPT_THREEPASS_MIN_LOG2, prev)
    assert rel_l2(a, b) <= tol(n, np.float32)


def test_three_pass_real_forward():
    import jtransforms_gb300 as J
    n = 1 << 23  # half-length complex FFT of 2^22 points: three passes
    x = np.random.default_rng(9).standard_normal(n).astype(np.float32)
    a = x.copy()
    J.FloatFFT_1D(n).realForward(a)
    spec = np.fft.rfft(x.astype(np.float64))
    want = np.empty(n)
    want[0::2] = spec.real[: n // 2]
    want[1::2] = spec.imag[: n // 2]
    want[1] = spec.real[n // 2]
    assert rel_l2(a, want) <= tol(n, np.float32)
