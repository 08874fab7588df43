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
    # (precision, n, batch): two-pass lengths use the scratch, 4096 is one pass;
    # f32 2^22 and f64 2^21 need exactly the whole 32 MiB per transform
    ("f32", 1 << 20, 6),
    ("f32", 1 << 14, 40),
    ("f64", 1 << 18, 3),
    ("f32", 4096, 16),
    ("f32", 1 << 22, 2),
    ("f64", 1 << 21, 2),
]


def _compare(plan, n, batch, dt, prec, inplace=False):
    """Two calls in a row of the no-allocation entry point against
    jt_execute_device, forward and scaled inverse.  Tolerance: relative L2 <=
    4 * eps * log2(n) of the precision."""
    import torch

    from jtransforms_gb300 import _native as N

    lib = N.load()
    g = torch.Generator(device="cuda").manual_seed(20110602 + n)
    x = torch.randn(2 * n * batch, dtype=dt, device="cuda", generator=g)
    stream = torch.cuda.current_stream()
    for op, scale in ((N.COMPLEX_FORWARD, 0), (N.COMPLEX_INVERSE, 1)):
        ref = x.clone()
        plan.execute(op, ref, 0, bool(scale), batch=batch, dist=2 * n)
        for _ in range(2):
            if inplace:
                out = x.clone()
                src = out
            else:
                out = torch.full_like(x, float("nan"))
                src = x
            rc = lib.jt_execute_device_noalloc(plan.handle, op, ctypes.c_void_p(src.data_ptr()),
                                               ctypes.c_void_p(out.data_ptr()), batch, scale,
                                               ctypes.c_void_p(stream.cuda_stream))
            assert rc == N.OK, N.strerror(rc)
            torch.cuda.synchronize()
            assert lib.jt_check_error() == N.OK
            err = rel_l2(out.cpu().numpy(), ref.cpu().numpy())
            assert err <= tol(n, np.float32 if prec == "f32" else np.float64), err


@pytest.mark.parametrize("prec,n,batch", CASES)
def test_noalloc_matches_regular_entry(prec, n, batch):
    import torch

    from jtransforms_gb300 import _native as N

    dt = torch.float32 if prec == "f32" else torch.float64
    plan = N.Plan(N.FFT, N.FLOAT32 if prec == "f32" else N.FLOAT64, [n])
    _compare(plan, n, batch, dt, prec)


@pytest.mark.parametrize("prec,n,batch", [("f32", 1 << 20, 3), ("f64", 4096, 8)])
def test_noalloc_in_place(prec, n, batch):
    """dev_in == dev_out, as the header allows."""
    import torch

    from jtransforms_gb300 import _native as N

    dt = torch.float32 if prec == "f32" else torch.float64
    plan = N.Plan(N.FFT, N.FLOAT32 if prec == "f32" else N.FLOAT64, [n])
    _compare(plan, n, batch, dt, prec, inplace=True)


def test_noalloc_three_pass():
    """A three-pass split (forced) draws one transform's scratch too."""
    import torch

    from jtransforms_gb300 import _native as N

    lib = N.load()
    n = 1 << 21
    assert lib.jt_set_split(N.FLOAT32, 21, 7, 7, 7) == N.OK
    try:
        plan = N.Plan(N.FFT, N.FLOAT32, [n])
    finally:
        lib.jt_set_split(N.FLOAT32, 21, -1, 0, 0)
    assert plan.algorithm(0) == 4
    _compare(plan, n, 3, torch.float32, "f32")


def test_noalloc_tensor_core_mode_runs_the_same_kernels():
    """A plan in the split tensor-core mode gives the same bits through both
    entry points."""
    import torch

    from jtransforms_gb300 import _native as N

    lib = N.load()
    n, batch = 1024, 64
    plan = N.Plan(N.FFT, N.FLOAT32, [n])
    plan.set_mode(N.MODE_TC_SPLIT)
    g = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randn(2 * n * batch, dtype=torch.float32, device="cuda", generator=g)
    ref = x.clone()
    plan.execute(N.COMPLEX_FORWARD, ref, 0, False, batch=batch, dist=2 * n)
    out = torch.empty_like(x)
    rc = lib.jt_execute_device_noalloc(plan.handle, N.COMPLEX_FORWARD, ctypes.c_void_p(x.data_ptr()),
                                       ctypes.c_void_p(out.data_ptr()), batch, 0,
                                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.OK
    torch.cuda.synchronize()
    assert torch.equal(out, ref)


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
