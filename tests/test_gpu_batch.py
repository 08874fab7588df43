"""GPU tests of the mixed-size batch (jt_batch_*): one persistent launch
over transforms of different sizes, algorithms and kinds must give the
results of running each transform on its own, and the oracle's."""
import numpy as np
import pytest

from tests._helpers import rel_l2, tol

pytestmark = pytest.mark.gpu

# (kind, precision, op, scale, sizes): the batch workload's kinds plus the
# inverse ops, over powers of two, 7-smooth lengths, primes on both sides of
# the Bluestein switch and lengths that take the two-pass path
ITEMS = [
    ("fft", "f32", "cf", False, [16, 64, 1024, 4096, 8192, 16384, 65536, 100, 360, 3000, 17, 211, 997, 4099, 65521]),
    ("fft", "f32", "ci", True, [32, 2048, 105, 1009, 32768]),
    ("fft", "f32", "rf", False, [16, 256, 8192, 32768, 65536, 120, 2310, 31, 509, 7919]),
    ("fft", "f64", "cf", False, [512, 8192, 16384, 99, 101]),
    ("fft", "f64", "ri", True, [64, 1000, 4096, 63]),
    ("dct", "f64", "fwd", True, [16, 1024, 8192, 16384, 65536, 100, 6000, 13, 211, 4093]),
    ("dct", "f64", "inv", True, [128, 360, 8192]),
    ("dst", "f64", "fwd", True, [64, 300]),
    ("dht", "f32", "fwd", False, [128, 1000]),
    # one-step forms: packed real inverse, DHT, DST inverse and DCT of even
    # lengths whose half length is mixed-radix, Bluestein inverses
    ("fft", "f32", "ri", True, [128, 2048, 210, 97]),
    ("dht", "f64", "fwd", False, [64, 210, 101]),
    ("dst", "f32", "inv", True, [32, 210, 4096]),
    ("fft", "f64", "ci", True, [97, 1021]),
    ("dct", "f32", "fwd", True, [210, 1024, 7]),
    # primes whose Bluestein convolution is too long for one task: separate
    # steps over a 7-smooth convolution (12289: a two-pass 24576-point one)
    ("fft", "f32", "cf", False, [4481, 12289]),
    ("fft", "f32", "rf", False, [4801]),
    ("fft", "f64", "ci", True, [2251]),
    ("dct", "f64", "fwd", True, [2521]),
]


def _setup():
    import torch

    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N

    opmap = {"cf": N.COMPLEX_FORWARD, "ci": N.COMPLEX_INVERSE, "rf": N.REAL_FORWARD, "ri": N.REAL_INVERSE,
             "fwd": N.FORWARD, "inv": N.INVERSE}
    kindmap = {"fft": N.FFT, "dct": N.DCT, "dst": N.DST, "dht": N.DHT}
    rng = np.random.default_rng(7)
    items, specs = [], []
    for kind, prec, op, scale, sizes in ITEMS:
        for n in sizes:
            plan = N.Plan(kindmap[kind], N.FLOAT32 if prec == "f32" else N.FLOAT64, [n])
            code = opmap[op]
            ext = plan.extent(code)
            dt = torch.float32 if prec == "f32" else torch.float64
            x = torch.from_numpy(rng.uniform(-1, 1, ext + (ext & 1))).to(dt).cuda()
            items.append((plan, code, x, scale))
            specs.append((kind, prec, code, scale, n, ext))
    return items, specs


def test_batch_matches_single_transforms_and_oracle(oracle):
    import torch

    from jtransforms_gb300 import _native as N

    items, specs = _setup()
    pristine = [it[2].clone() for it in items]
    batch = N.Batch(items)
    # reference: each transform on its own through the regular path
    ref = []
    for (plan, code, x, scale), p0 in zip(items, pristine):
        y = p0.clone()
        plan.execute(code, y, 0, scale)
        ref.append(y)
    for mode in ("run", "run_graph", "run_graph"):
        for it, p0 in zip(items, pristine):
            it[2].copy_(p0)
        getattr(batch, mode)()
        torch.cuda.synchronize()
        for (plan, code, x, scale), y, (kind, prec, _, _, n, ext) in zip(items, ref, specs):
            dt = np.float32 if prec == "f32" else np.float64
            err = rel_l2(x[:ext].cpu().numpy(), y[:ext].cpu().numpy())
            assert err <= tol(n, dt), (mode, kind, prec, code, n, err)
    # a spot check of the batch output against the oracle
    kmap = {"fft": oracle.FFT, "dct": oracle.DCT, "dst": oracle.DST, "dht": oracle.DHT}
    for (plan, code, x, scale), p0, (kind, prec, _, _, n, ext) in list(zip(items, pristine, specs))[::3]:
        a = p0[:ext].cpu().numpy().copy()
        oracle.run(kmap[kind], code, [n], a, scale)
        dt = np.float32 if prec == "f32" else np.float64
        assert rel_l2(x[:ext].cpu().numpy(), a) <= tol(n, dt), (kind, prec, code, n)


def test_batch_per_transform_baseline():
    import torch

    from jtransforms_gb300 import _native as N

    items, specs = _setup()
    pristine = [it[2].clone() for it in items]
    batch = N.Batch(items)
    batch.run()
    torch.cuda.synchronize()
    first = [it[2].clone() for it in items]
    for it, p0 in zip(items, pristine):
        it[2].copy_(p0)
    batch.run_per_transform()
    torch.cuda.synchronize()
    for (plan, code, x, scale), f, (kind, prec, _, _, n, ext) in zip(items, first, specs):
        dt = np.float32 if prec == "f32" else np.float64
        assert rel_l2(x[:ext].cpu().numpy(), f[:ext].cpu().numpy()) <= tol(n, dt)
