"""GPU test of jt_execute_device_noalloc, the complex FFT entry point that
allocates nothing (for callers that cannot allocate device memory when they
transform, e.g. inside CUDA stream capture).  It must give the same result as
the regular jt_execute_device on the same input, on two calls in a row (the
second call reuses the shared scratch array the first one left behind).

Named to be collected last, so a run that stops at the first failure has run
every other test before it."""
import ctypes

import numpy as np
import pytest

from tests._helpers import rel_l2, tol

pytestmark = pytest.mark.gpu

CASES = [
    # (precision, n, batch): two-pass lengths use the scratch, 4096 is one pass
    ("f32", 1 << 20, 6),
    ("f32", 1 << 14, 40),
    ("f64", 1 << 18, 3),
    ("f32", 4096, 16),
]


@pytest.mark.parametrize("prec,n,batch", CASES)
def test_noalloc_matches_regular_entry(prec, n, batch):
    import torch

    from jtransforms_gb300 import _native as N

    lib = N.load()
    dt = torch.float32 if prec == "f32" else torch.float64
    plan = N.Plan(N.FFT, N.FLOAT32 if prec == "f32" else N.FLOAT64, [n])
    g = torch.Generator(device="cuda").manual_seed(20110602 + n)
    x = torch.randn(2 * n * batch, dtype=dt, device="cuda", generator=g)
    stream = torch.cuda.current_stream()
    for op, scale in ((N.COMPLEX_FORWARD, 0), (N.COMPLEX_INVERSE, 1)):
        ref = x.clone()
        plan.execute(op, ref, 0, bool(scale), batch=batch, dist=2 * n)
        for _ in range(2):
            out = torch.full_like(x, float("nan"))
            rc = lib.jt_execute_device_noalloc(plan.handle, op, ctypes.c_void_p(x.data_ptr()),
                                               ctypes.c_void_p(out.data_ptr()), batch, scale,
                                               ctypes.c_void_p(stream.cuda_stream))
            assert rc == N.OK, N.strerror(rc)
            torch.cuda.synchronize()
            err = rel_l2(out.cpu().numpy(), ref.cpu().numpy())
            assert err <= tol(n, np.float32 if prec == "f32" else np.float64), err


def test_noalloc_rejects_beyond_scratch():
    from jtransforms_gb300 import _native as N

    lib = N.load()
    big = N.Plan(N.FFT, N.FLOAT32, [1 << 23])  # two-pass, needs 64 MiB of scratch
    rc = lib.jt_execute_device_noalloc(big.handle, N.COMPLEX_FORWARD, ctypes.c_void_p(256), ctypes.c_void_p(256), 1, 0,
                                       None)
    assert rc == N.ESCRATCH
    blue = N.Plan(N.FFT, N.FLOAT32, [10158])  # Bluestein length
    rc = lib.jt_execute_device_noalloc(blue.handle, N.COMPLEX_FORWARD, ctypes.c_void_p(256), ctypes.c_void_p(256), 1, 0,
                                       None)
    assert rc == N.ESCRATCH
