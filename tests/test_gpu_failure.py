"""Failure paths and plan setup, on the GPU without faulting it.

* A bounded device wait that runs out: the batch kernel's dependency waits
  are given a short poll limit, and a test hook makes every transform's
  first step wait on a step that never runs (a flag nothing sets).  The
  kernel gives up, raises the library's error flag and returns; the host
  reads JT_ETIMEOUT, and the context stays usable (the same batch then runs
  correctly).  The reference logs a failed worker instead
  (fft/DoubleFFT_1D.java:711-715); here the status reaches the caller.
* A device allocation that fails: a scratch budget smaller than the call
  needs gives JT_ENOMEM before anything launches, which the Java-mirror
  classes raise as IllegalStateException.
* The table cache: a second plan of the same kind and size builds no tables
  (no table kernel launches), as the reference builds them once per object
  (fft/DoubleFFT_1D.java:128-156).
"""
import numpy as np
import pytest

from tests._helpers import rel_l2, tol

pytestmark = pytest.mark.gpu


def _batch_items(rng):
    import torch

    from jtransforms_gb300 import _native as N
    items, refs = [], []
    for n, kind, prec in ((256, N.FFT, N.FLOAT32), (1000, N.FFT, N.FLOAT32), (211, N.FFT, N.FLOAT64),
                          (4096, N.FFT, N.FLOAT32)):
        p = N.Plan(kind, prec, [n])
        dt = torch.float32 if prec == N.FLOAT32 else torch.float64
        x = torch.from_numpy(rng.uniform(-1, 1, 2 * n)).to(dt).cuda()
        ref = x.clone()
        p.execute(N.COMPLEX_FORWARD, ref)
        items.append((p, N.COMPLEX_FORWARD, x, False))
        refs.append((x.clone(), ref))
    return items, refs


def test_batch_wait_runs_out_and_reports_timeout():
    import torch

    from jtransforms_gb300 import _native as N
    lib = N.load()
    rng = np.random.default_rng(3)
    items, refs = _batch_items(rng)
    torch.cuda.synchronize()
    assert lib.jt_check_error() == N.OK
    prev_polls = N.set_option(N.OPT_BATCH_WAIT_POLLS, 256)
    prev_hook = N.set_option(N.OPT_BATCH_STALL_TEST, 1)
    try:
        stalled = N.Batch(items)
    finally:
        N.set_option(N.OPT_BATCH_STALL_TEST, prev_hook)
        N.set_option(N.OPT_BATCH_WAIT_POLLS, prev_polls)
    stalled.run()
    torch.cuda.synchronize()  # the kernel returned: its waits are bounded
    assert lib.jt_check_error() == N.ETIMEOUT
    assert lib.jt_check_error() == N.OK  # reading clears the flag
    # the context is still usable: a normal batch over fresh inputs is right
    for (p, op, x, s), (x0, _) in zip(items, refs):
        x.copy_(x0)
    good = N.Batch(items)
    good.run()
    torch.cuda.synchronize()
    assert lib.jt_synchronize() == N.OK
    for (p, op, x, s), (_, ref) in zip(items, refs):
        eps = np.float32 if x.dtype == torch.float32 else np.float64
        assert rel_l2(x.cpu().numpy(), ref.cpu().numpy()) <= tol(x.numel() // 2, eps)


def test_scratch_budget_gives_enomem_then_recovers():
    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    n = 1 << 21  # packed real transform on a host array: 8 MiB ring buffers at least
    f = J.FloatFFT_1D(n)
    x = np.random.default_rng(5).standard_normal(n).astype(np.float32)
    a = x.copy()
    prev = N.set_option(N.OPT_ARENA_LIMIT_MB, 1)
    try:
        with pytest.raises(J.IllegalStateException):
            f.realForward(a)
    finally:
        N.set_option(N.OPT_ARENA_LIMIT_MB, prev)
    assert np.array_equal(a, x)  # nothing ran
    f.realForward(a)
    spec = np.fft.rfft(x.astype(np.float64))
    want = np.empty(n)
    want[0::2] = spec.real[: n // 2]
    want[1::2] = spec.imag[: n // 2]
    want[1] = spec.real[n // 2]
    assert rel_l2(a, want) <= tol(n, np.float32)


@pytest.mark.parametrize("cls,n", [("DoubleFFT_1D", 3003), ("FloatFFT_1D", 3 * 5 * 7 * 11 * 13),
                                   ("DoubleDCT_1D", 1155), ("DoubleFFT_3D", (6, 10, 14))])
def test_second_plan_builds_no_tables(cls, n):
    import jtransforms_gb300 as J
    dims = n if isinstance(n, tuple) else (n,)
    J.launch_count(reset=True)
    first = getattr(J, cls)(*dims)
    built = J.launch_count(reset=True)
    assert built > 0  # sizes no other test uses: the first plan builds its tables
    second = getattr(J, cls)(*dims)
    assert J.launch_count(reset=True) == 0
    # both plans transform alike
    N = int(np.prod(dims))
    ext = 2 * N if cls.endswith(("FFT_1D", "FFT_3D")) else N
    dt = np.float32 if cls.startswith("Float") else np.float64
    x = np.random.default_rng(1).uniform(-1, 1, ext).astype(dt)
    a, b = x.copy(), x.copy()
    if "FFT" in cls:
        first.complexForward(a)
        second.complexForward(b)
    else:
        first.forward(a, True)
        second.forward(b, True)
    assert np.array_equal(a, b)
    del first, second
