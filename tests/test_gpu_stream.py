"""Host-staged four-step: a complex 1D transform whose device working set
exceeds the device budget streams through host pieces (the LargeArray path
of fft/DoubleFFT_1D.java:280-304 for arrays the device cannot hold).  The
budget is lowered with JT_OPT_ARENA_LIMIT_MB so that moderate lengths take
this path, and the results are checked against an FP64 FFT of the same
input, with offsets and batches.  Tolerance: relative L2 <= 4 * eps *
log2(n) of the precision."""
import numpy as np
import pytest

from tests._helpers import rel_l2, tol

pytestmark = pytest.mark.gpu


def _fp64(x, n, inverse=False, scale=False):
    z = x.astype(np.float64).reshape(-1, n, 2)
    c = z[..., 0] + 1j * z[..., 1]
    y = (np.fft.ifft(c, axis=1) * (1 if scale else n)) if inverse else np.fft.fft(c, axis=1)
    out = np.empty(x.size)
    out[0::2] = y.real.ravel()
    out[1::2] = y.imag.ravel()
    return out


# (class, log2 n, budget MiB, batch, offset in scalars)
CASES = [("FloatFFT_1D", 22, 8, 1, 0), ("FloatFFT_1D", 22, 8, 2, 1), ("DoubleFFT_1D", 20, 4, 1, 3),
         ("FloatFFT_1D", 24, 32, 1, 0), ("DoubleFFT_1D", 21, 2, 2, 0)]


@pytest.mark.parametrize("cls,lg,mb,batch,off", CASES)
def test_streamed_four_step_matches_fp64(cls, lg, mb, batch, off):
    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    n = 1 << lg
    dt = np.float32 if cls.startswith("Float") else np.float64
    f = getattr(J, cls)(n)
    assert f.plan.algorithm(0) in (1, 4)
    rng = np.random.default_rng(lg + mb)
    x = rng.standard_normal(2 * n * batch).astype(dt)
    a = np.concatenate([np.zeros(off, dt), x])
    prev = N.set_option(N.OPT_ARENA_LIMIT_MB, mb)
    try:
        J.launch_count(reset=True)
        f.plan.execute(N.COMPLEX_FORWARD, a, off, False, batch=batch, dist=2 * n)
        assert J.launch_count() > 0
        got = a[off:].copy()
        assert rel_l2(got, _fp64(x, n)) <= tol(n, dt)
        a[off:] = x
        f.plan.execute(N.COMPLEX_INVERSE, a, off, True, batch=batch, dist=2 * n)
        assert rel_l2(a[off:], _fp64(x, n, inverse=True, scale=True)) <= tol(n, dt)
        assert not a[:off].any()
    finally:
        N.set_option(N.OPT_ARENA_LIMIT_MB, prev)
    # the same call without the budget (one device pass) agrees
    b = np.concatenate([np.zeros(off, dt), x])
    f.plan.execute(N.COMPLEX_FORWARD, b, off, False, batch=batch, dist=2 * n)
    assert rel_l2(got, b[off:]) <= tol(n, dt)


def test_budget_too_small_for_a_real_transform():
    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    n = 1 << 22
    a = np.random.default_rng(2).standard_normal(n).astype(np.float32)
    prev = N.set_option(N.OPT_ARENA_LIMIT_MB, 4)
    try:
        with pytest.raises(J.IllegalStateException):
            J.FloatFFT_1D(n).realForward(a)  # packed real ops do not stream
    finally:
        N.set_option(N.OPT_ARENA_LIMIT_MB, prev)
