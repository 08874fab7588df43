"""GPU parity of 1D lengths beyond one plan's earlier reach: the reference's
LargeArray lengths (fft/DoubleFFT_1D.java:280-304, the useLargeArrays switch
at :122), where n = 2^31 complex floats is 2^32 array elements.

* Double powers of two above 4096 x 4096 run three register passes, and
  double Bluestein lengths now pad to more than 2^24. Both are checked
  against an FP64 FFT of the same input.
* 2^31 complex floats (16 GiB), 2^30 complex doubles and a float
  Bluestein length of 2^26 + 1 are checked through size-independent
  properties computed on the device:
  - a single tone e^{2 pi i k0 j / n} transforms to n at bin k0 and zero
    elsewhere;
  - forward then scaled inverse returns the input.

Tolerance: relative L2 <= 4 * eps * log2(n) of the precision.
"""
import math

import numpy as np
import pytest

from tests._helpers import rel_l2, tol

pytestmark = pytest.mark.gpu


def _fp64_fft(x, n):
    z = x.astype(np.float64).reshape(-1, n, 2)
    y = np.fft.fft(z[..., 0] + 1j * z[..., 1], axis=1)
    out = np.empty(x.size)
    out[0::2] = y.real.ravel()
    out[1::2] = y.imag.ravel()
    return out


@pytest.mark.parametrize("cls,n", [("DoubleFFT_1D", 1 << 25), ("DoubleFFT_1D", (1 << 24) + 3)])
def test_large_lengths_against_fp64(cls, n):
    import jtransforms_gb300 as J
    f = getattr(J, cls)(n)
    assert f.plan.algorithm(0) == (4 if n & (n - 1) == 0 else 2)  # three passes / Bluestein
    dt = np.float64 if cls.startswith("Double") else np.float32
    x = np.random.default_rng(n % 1000).standard_normal(2 * n).astype(dt)
    a = x.copy()
    f.complexForward(a)
    assert rel_l2(a, _fp64_fft(x, n)) <= tol(n, dt)
    f.complexInverse(a, True)
    assert rel_l2(a, x) <= tol(n, dt)


def _tone(n, k0, dtype):
    """Interleaved e^{2 pi i k0 j / n}, j < n, built on the device in chunks
    (the exponent reduced exactly in 64-bit integers)."""
    import torch
    x = torch.empty(2 * n, dtype=dtype, device="cuda")
    step = 1 << 27
    for j0 in range(0, n, step):
        j = torch.arange(j0, min(n, j0 + step), dtype=torch.int64, device="cuda")
        ang = ((j * k0) % n).to(torch.float64) * (2.0 * math.pi / n)
        v = x[2 * j0:2 * (j0 + j.numel())].view(-1, 2)
        v[:, 0] = torch.cos(ang).to(dtype)
        v[:, 1] = torch.sin(ang).to(dtype)
    return x


def _tone_error(y, n, k0):
    """||y - n e_{k0}||_2 / n, reduced on the device in chunks."""
    import torch
    acc = 0.0
    step = 1 << 28
    for i0 in range(0, 2 * n, step):
        acc += float(torch.sum(y[i0:i0 + step].to(torch.float64) ** 2))
    re, im = float(y[2 * k0]), float(y[2 * k0 + 1])
    acc += (re - n) ** 2 - re * re
    return math.sqrt(max(acc, 0.0)) / n


@pytest.mark.parametrize("cls,n,algo", [("FloatFFT_1D", 1 << 31, 4), ("DoubleFFT_1D", 1 << 30, 4),
                                        ("FloatFFT_1D", (1 << 26) + 1, 2)])
def test_huge_single_tone_and_round_trip(cls, n, algo):
    import torch

    import jtransforms_gb300 as J
    f = getattr(J, cls)(n)
    assert f.plan.algorithm(0) == algo  # three passes / Bluestein padded to 2^28
    dt = torch.float32 if cls.startswith("Float") else torch.float64
    npdt = np.float32 if dt == torch.float32 else np.float64
    k0 = 123456789 % n
    x = _tone(n, k0, dt)
    f.complexForward(x)
    torch.cuda.synchronize()
    assert _tone_error(x, n, k0) <= tol(n, npdt)
    # the scaled inverse brings the tone back
    f.complexInverse(x, True)
    torch.cuda.synchronize()
    ref = _tone(n, k0, dt)
    num = 0.0
    step = 1 << 28
    for i0 in range(0, 2 * n, step):
        num += float(torch.sum((x[i0:i0 + step].to(torch.float64) - ref[i0:i0 + step].to(torch.float64)) ** 2))
    assert math.sqrt(num / n) <= tol(n, npdt)
    del x, ref
    torch.cuda.empty_cache()


def test_host_array_above_2_31_elements():
    """jt_execute on a HOST array of 2^32 floats (2^31 complex elements, the
    FloatLargeArray overload's range): the single tone comes out at bin k0
    and the scaled inverse brings it back."""
    import torch

    import jtransforms_gb300 as J
    n = 1 << 31
    f = J.FloatFFT_1D(n)
    k0 = 987654321 % n
    host = _tone(n, k0, torch.float32).cpu().numpy()
    assert host.size == 1 << 32
    f.complexForward(host)
    y = torch.from_numpy(host).cuda()
    assert _tone_error(y, n, k0) <= tol(n, np.float32)
    del y
    f.complexInverse(host, True)
    back = torch.from_numpy(host).cuda()
    ref = _tone(n, k0, torch.float32)
    num = 0.0
    step = 1 << 28
    for i0 in range(0, 2 * n, step):
        num += float(torch.sum((back[i0:i0 + step].to(torch.float64) - ref[i0:i0 + step].to(torch.float64)) ** 2))
    assert math.sqrt(num / n) <= tol(n, np.float32)
    del back, ref, host
    torch.cuda.empty_cache()
