"""GPU: the mixed-radix tile kernel in each of its four pass orders
(JT_OPT_RADIX_ORDER: power-of-two or odd radices first, 16s or 8s for the
power of two) gives the DFT within the reference's tolerance, for complex
and real lines in both precisions. The autotuned table picks one order per
size class; every order must be correct for that choice to be free."""
import numpy as np
import pytest

from tests._helpers import rel_l2, tol

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order", [0, 1, 2, 3])
@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n", [12, 96, 360, 1000, 2310, 3584])
def test_tile_orders(order, prec, n):
    import torch
    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    dt = np.float64 if prec == "f64" else np.float32
    prev = N.set_option(N.OPT_RADIX_ORDER, order)
    try:
        cls = J.FloatFFT_1D if prec == "f32" else J.DoubleFFT_1D
        f = cls(n)
        assert f.plan.algorithm(0) == 0  # one tile pass
        batch = 9
        rng = np.random.default_rng(n + order)
        x = rng.uniform(-1, 1, (batch, 2 * n))
        dev = torch.from_numpy(x.astype(dt).ravel().copy()).cuda()
        f.plan.execute(N.COMPLEX_FORWARD, dev, 0, False, batch=batch, dist=2 * n)
        got = dev.cpu().numpy().astype(np.float64).reshape(batch, 2 * n)
        z = x.astype(dt).astype(np.float64)
        y = np.fft.fft(z[:, 0::2] + 1j * z[:, 1::2], axis=1)
        want = np.empty_like(got)
        want[:, 0::2], want[:, 1::2] = y.real, y.imag
        assert rel_l2(got, want) <= tol(n, dt)
        # realForward then realInverse(scale) returns the input
        r = rng.uniform(-1, 1, (batch, n))
        rd = torch.from_numpy(r.astype(dt).ravel().copy()).cuda()
        f.plan.execute(N.REAL_FORWARD, rd, 0, False, batch=batch, dist=n)
        f.plan.execute(N.REAL_INVERSE, rd, 0, True, batch=batch, dist=n)
        assert rel_l2(rd.cpu().numpy().reshape(batch, n), r.astype(dt)) <= 2 * tol(n, dt)
    finally:
        N.set_option(N.OPT_RADIX_ORDER, prev)
