"""Plans, threads and the table cache on the GPU.

* Several host threads transform at once, each with its own plans and some
  sharing one plan: every result matches FP64 (the C ABI serialises a plan's
  host work under its mutex and gives each calling thread its own stream).
* A plan destroyed while its kernels are still queued: the kernels finish
  correctly, because destroying a plan frees no tables (they stay in the
  table cache) and synchronises nothing.
* More distinct plans than the cache keeps idle: entries are evicted (the
  device is synchronised first), and plans created afterwards rebuild what
  they need and transform correctly.
Tolerance: relative L2 <= 4 * eps * log2(n) of the precision against numpy's
FP64 FFT."""
import threading

import numpy as np
import pytest

from tests._helpers import rel_l2, tol

pytestmark = pytest.mark.gpu


def _fft64(x):
    z = x.astype(np.float64).reshape(-1, 2)
    return np.fft.fft(z[:, 0] + 1j * z[:, 1])


def _as_complex(a):
    z = a.astype(np.float64).reshape(-1, 2)
    return z[:, 0] + 1j * z[:, 1]


def test_concurrent_host_threads():
    import jtransforms_gb300 as J
    shared = J.FloatFFT_1D(4096)
    errors = []

    def work(tid):
        try:
            rng = np.random.default_rng(100 + tid)
            own = (J.DoubleFFT_1D if tid % 2 else J.FloatFFT_1D)(1000 + 24 * tid)
            for it in range(6):
                for f, n, dt in ((own, own.plan.dims[0], own.plan.dtype), (shared, 4096, np.float32)):
                    x = rng.standard_normal(2 * n).astype(dt)
                    a = x.copy()
                    f.complexForward(a)
                    err = rel_l2(_as_complex(a), _fft64(x))
                    if err > tol(n, dt):
                        errors.append((tid, it, n, err))
        except Exception as e:  # reported below
            errors.append((tid, repr(e)))

    th = [threading.Thread(target=work, args=(t,)) for t in range(6)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors


def test_destroy_with_kernels_in_flight():
    import torch

    from jtransforms_gb300 import _native as N
    n, batch = 1 << 20, 16  # two-pass length, several long launches
    x = torch.randn(2 * n * batch, dtype=torch.float32, device="cuda")
    want = x.clone()
    keep = N.Plan(N.FFT, N.FLOAT32, [n])  # reference result through a plan that stays alive
    keep.execute(N.COMPLEX_FORWARD, want, 0, False, batch=batch, dist=2 * n)
    torch.cuda.synchronize()
    p = N.Plan(N.FFT, N.FLOAT32, [n])
    y = x.clone()
    p.execute(N.COMPLEX_FORWARD, y, 0, False, batch=batch, dist=2 * n)
    p.__del__()  # jt_plan_destroy while the launches may still run
    torch.cuda.synchronize()
    assert torch.equal(y, want)


def test_cache_eviction_and_rebuild():
    import jtransforms_gb300 as J
    # 40 distinct lengths, each plan destroyed at once: the cache keeps 32
    # idle entries per object type and evicts the rest
    for k in range(40):
        f = J.FloatFFT_1D(2 * (1009 + 2 * k))
        del f
    for n in (2018, 2096, 4096):
        f = J.FloatFFT_1D(n)
        x = np.random.default_rng(n).standard_normal(2 * n).astype(np.float32)
        a = x.copy()
        f.complexForward(a)
        assert rel_l2(_as_complex(a), _fft64(x)) <= tol(n, np.float32)
