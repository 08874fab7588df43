"""GPU: the one-kernel DCT/DST/DHT and real lines load their input two ways,
and Float packed real lines run in either of their two forms.

Contiguous lines whose scalar pairs (2j, 2j+1) are aligned complex values
are loaded as pairs: straight into registers when 16 or more threads share a
line (n = 1024), through a coalesced staged block when fewer do (n = 64).
Lines at an odd scalar offset are loaded one scalar at a time. Both must give
the transform the reference defines (dct/DoubleDCT_1D.java:169-243,
dst/DoubleDST_1D.java, dht/DoubleDHT_1D.java), checked here against SciPy in
FP64 on a device batch at offset 0 and at offset 1.
"""
import numpy as np
import pytest

from tests._helpers import rel_l2, tol

pytestmark = pytest.mark.gpu


def _want(kind, op, x):
    import scipy.fft as sfft
    if kind == "dht":
        f = np.fft.fft(x, axis=-1)
        return f.real - f.imag
    t = sfft.dct if kind == "dct" else sfft.dst
    if op == "fwd":
        return t(x, type=2, norm="ortho", axis=-1)
    return t(x, type=3, norm="ortho", axis=-1)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("kind,op", [("dct", "fwd"), ("dct", "inv"), ("dst", "fwd"), ("dht", "fwd")])
@pytest.mark.parametrize("n", [64, 1024])
@pytest.mark.parametrize("off", [0, 1])
def test_r2r_lines_paired_and_scalar_loads(prec, kind, op, n, off):
    import torch
    from jtransforms_gb300 import _native as N
    dt = np.float64 if prec == "f64" else np.float32
    kcode = {"dct": N.DCT, "dst": N.DST, "dht": N.DHT}[kind]
    plan = N.Plan(kcode, N.FLOAT32 if prec == "f32" else N.FLOAT64, [n])
    batch = 37
    rng = np.random.default_rng(n + off)
    x = rng.uniform(-1, 1, (batch, n))
    buf = np.full(off + batch * n + 3, 5.0)
    buf[off:off + batch * n] = x.ravel()
    dev = torch.from_numpy(buf.astype(dt)).cuda()
    scale = kind != "dht"
    plan.execute(N.FORWARD if op == "fwd" else N.INVERSE, dev, off, scale, batch=batch, dist=n)
    got = dev.cpu().numpy().astype(np.float64)
    want = _want(kind, op, x.astype(dt).astype(np.float64))
    assert rel_l2(got[off:off + batch * n].reshape(batch, n), want) <= tol(n, dt)
    # the elements around the batch are untouched
    assert np.all(got[:off] == 5.0) and np.all(got[off + batch * n:] == 5.0)


@pytest.mark.parametrize("fused", [1, 0])
@pytest.mark.parametrize("n", [32, 256, 2048, 8192])
def test_float_real_lines_both_forms(fused, n):
    """Float packed realForward / realInverse of power-of-two lines run as one
    kernel (JT_OPT_REAL_FUSED_F32 = 1, the default) or as the pipelined FFT
    and a separate split (0); both give numpy's spectrum in the packed layout
    (fft/DoubleFFT_1D.java:433-451) and return the input."""
    import torch
    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    prev = N.set_option(N.OPT_REAL_FUSED_F32, fused)
    try:
        f = J.FloatFFT_1D(n)
        batch = 33
        rng = np.random.default_rng(n + fused)
        x = rng.uniform(-1, 1, (batch, n)).astype(np.float32)
        dev = torch.from_numpy(x.ravel().copy()).cuda()
        f.plan.execute(N.REAL_FORWARD, dev, 0, False, batch=batch, dist=n)
        got = dev.cpu().numpy().astype(np.float64).reshape(batch, n)
        F = np.fft.rfft(x.astype(np.float64), axis=1)
        want = np.empty((batch, n))
        want[:, 0] = F[:, 0].real
        want[:, 1] = F[:, n // 2].real
        want[:, 2::2] = F[:, 1:n // 2].real
        want[:, 3::2] = F[:, 1:n // 2].imag
        assert rel_l2(got, want) <= tol(n, np.float32)
        f.plan.execute(N.REAL_INVERSE, dev, 0, True, batch=batch, dist=n)
        assert rel_l2(dev.cpu().numpy().reshape(batch, n), x) <= 2 * tol(n, np.float32)
    finally:
        N.set_option(N.OPT_REAL_FUSED_F32, prev)
