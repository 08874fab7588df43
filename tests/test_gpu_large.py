"""GPU parity of the pass splits of large Float lengths: the compiled plan
table's choice (two or three passes) and every split kind forced through
jt_set_split, against an FP64 FFT of the same input; realForward of a length
whose half-length FFT runs three passes.  Tolerance: relative L2 <=
4 * eps_float * log2(n) against FP64."""
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


def _check(f, n, batch, seed):
    from jtransforms_gb300 import _native as N
    x = np.random.default_rng(seed).standard_normal(2 * n * batch).astype(np.float32)
    a = x.copy()
    f.plan.execute(N.COMPLEX_FORWARD, a, 0, False, batch=batch, dist=2 * n)
    assert rel_l2(a, _fp64_fft(x, n)) <= tol(n, np.float32)
    for s in (True, False):
        c = x.copy()
        f.plan.execute(N.COMPLEX_INVERSE, c, 0, s, batch=batch, dist=2 * n)
        assert rel_l2(c, _fp64_fft(x, n, inverse=True, scale=s)) <= tol(n, np.float32)


@pytest.mark.parametrize("lg,batch", [(21, 2), (22, 1), (23, 1), (24, 1)])
def test_table_split_large(lg, batch):
    import jtransforms_gb300 as J
    f = J.FloatFFT_1D(1 << lg)
    assert f.plan.algorithm(0) in (1, 4)  # two or three passes
    _check(f, 1 << lg, batch, lg)


# one entry per split kind: one pass, two passes either way round, three
# passes with short and long first passes, lengths up to 4096 per pass
FORCED = [(14, (0, 0, 0), 0), (14, (4, 10, 0), 1), (16, (12, 4, 0), 1), (18, (9, 9, 0), 1), (18, (6, 6, 6), 4),
          (20, (4, 6, 10), 4), (21, (7, 7, 7), 4), (22, (11, 11, 0), 1), (22, (10, 6, 6), 4), (24, (12, 12, 0), 1)]


@pytest.mark.parametrize("lg,split,algo", FORCED)
def test_forced_split(lg, split, algo):
    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    lib = N.load()
    assert lib.jt_set_split(N.FLOAT32, lg, *split) == N.OK
    try:
        f = J.FloatFFT_1D(1 << lg)
    finally:
        lib.jt_set_split(N.FLOAT32, lg, -1, 0, 0)
    assert f.plan.algorithm(0) == algo
    _check(f, 1 << lg, 2 if lg <= 20 else 1, 100 + lg)


def test_set_split_rules():
    from jtransforms_gb300 import _native as N
    lib = N.load()
    assert lib.jt_set_split(N.FLOAT32, 20, 10, 9, 0) == N.EINVAL      # sums to 19
    assert lib.jt_set_split(N.FLOAT32, 26, 13, 13, 0) == N.EINVAL     # a pass above 4096
    assert lib.jt_set_split(N.FLOAT64, 24, 13, 6, 5) == N.EINVAL      # a pass above 4096
    assert lib.jt_set_split(N.FLOAT32, 31, 0, 0, 0) == N.EINVAL


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
