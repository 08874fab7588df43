"""GPU parity of the split-operand tensor-core mode (JT_MODE_TC_SPLIT) of
Float32 FFT plans: radix-16 stages as TF32 head/remainder products on the
tensor cores.  Bound: relative L2 <= 1e-6 against an FP64 FFT of the same
float32 input, on i.i.d. N(0,1) data (input set a) and on the 60 dB set
(8 unit complex exponentials + 1e-3 N(0,1), input set b); and the result
stays within 2e-6 of the plain FP32 mode."""
import numpy as np
import pytest

from tests._helpers import rel_l2

pytestmark = pytest.mark.gpu

TC_TOL = 1e-6
ROW_LENGTHS = [16, 32, 64, 128, 256, 512, 1024, 2048]


def _plan(n, tc):
    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    f = J.FloatFFT_1D(n)
    f.plan.set_mode(N.MODE_TC_SPLIT if tc else N.MODE_FP32)
    return f


def _set_a(n, batch, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(2 * n * batch).astype(np.float32)


def _set_b(n, batch, seed):
    rng = np.random.default_rng(seed)
    x = np.empty((batch, n), np.complex128)
    j = np.arange(n)
    for r in range(batch):
        bins = rng.integers(0, n, 8)
        ph = rng.uniform(0, 2 * np.pi, 8)
        x[r] = np.exp(1j * (2 * np.pi * np.outer(j, bins) / n + ph)).sum(1)
        x[r] += 1e-3 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    out = np.empty(2 * n * batch, np.float32)
    out[0::2] = x.real.ravel()
    out[1::2] = x.imag.ravel()
    return out


def _ref(x, n, inverse=False, scale=False):
    z = x.astype(np.float64).reshape(-1, n, 2)
    c = z[..., 0] + 1j * z[..., 1]
    y = np.fft.ifft(c, axis=1) * (1 if scale else n) if inverse else np.fft.fft(c, axis=1)
    out = np.empty(x.size, np.float64)
    out[0::2] = y.real.ravel()
    out[1::2] = y.imag.ravel()
    return out


def _run(f, x, n, batch, op):
    from jtransforms_gb300 import _native as N
    a = x.copy()
    if op == "cf":
        f.plan.execute(N.COMPLEX_FORWARD, a, 0, False, batch=batch, dist=2 * n)
    else:
        f.plan.execute(N.COMPLEX_INVERSE, a, 0, op == "ci_s", batch=batch, dist=2 * n)
    return a


@pytest.mark.parametrize("n", ROW_LENGTHS)
@pytest.mark.parametrize("op", ["cf", "ci_s", "ci_u"])
def test_tc_split_rows(n, op):
    # whole tiles of 2048 elements plus a ragged last tile
    batch = 3 * (2048 // n) + 1
    x = _set_a(n, batch, n)
    got = _run(_plan(n, True), x, n, batch, op)
    ref = _ref(x, n, inverse=op != "cf", scale=op == "ci_s")
    assert rel_l2(got, ref) <= TC_TOL
    plain = _run(_plan(n, False), x, n, batch, op)
    assert rel_l2(got, plain) <= 2 * TC_TOL
    # different arithmetic: the products really ran on the tensor cores
    assert not np.array_equal(got, plain)


@pytest.mark.parametrize("n", [256, 1024, 2048])
def test_tc_split_60db(n):
    batch = 2048 // n * 4
    x = _set_b(n, batch, 7 + n)
    got = _run(_plan(n, True), x, n, batch, "cf")
    assert rel_l2(got, _ref(x, n)) <= TC_TOL


@pytest.mark.parametrize("n", [1024, 16384, 1000, 4096 * 3])
def test_tc_split_other_paths(n):
    """Lengths whose passes are not row passes of 16..2048 (column passes,
    mixed radix, Bluestein) run the plain kernels under the mode; results
    still match FP64, and realForward goes through the mode too."""
    from jtransforms_gb300 import _native as N
    batch = 2
    x = _set_a(n, batch, 3)
    got = _run(_plan(n, True), x, n, batch, "cf")
    assert rel_l2(got, _ref(x, n)) <= 4e-6
    f = _plan(n, True)
    r = x[: n].copy()
    f.plan.execute(N.REAL_FORWARD, r, 0, False)
    spec = np.fft.fft(x[:n].astype(np.float64))
    if n % 2 == 0:
        want = np.empty(n)
        want[0::2] = spec.real[: n // 2]
        want[1::2] = spec.imag[: n // 2]
        want[1] = spec.real[n // 2]
        assert rel_l2(r, want) <= 4e-6


def test_tc_split_mode_rules():
    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    d = J.DoubleFFT_1D(1024)
    with pytest.raises(N.IllegalArgumentException):
        d.plan.set_mode(N.MODE_TC_SPLIT)
    f = J.FloatFFT_1D(1024)
    with pytest.raises(N.IllegalArgumentException):
        f.plan.set_mode(7)
