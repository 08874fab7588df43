"""The bench's multi-GPU path on CPU: two gloo ranks (replicas, weak
scaling) go through the same rank setup, start barrier and max-over-ranks
reduction as the NCCL ranks of `bench.py --gpus N`, each transforming its own
seeded batch with the oracle; and the reference arm's non-zero ranks exit
without work."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    from oracle import oracle as O
    w, r, local = bench.dist_setup(None)
    bench.dist_init(w, "gloo")
    bench.dist_barrier(w)
    # each rank its own batch (seed + rank), as the bench's replicas
    n, batch = 256, 8
    x = np.random.default_rng(bench.SEED + r).standard_normal(2 * n * batch).astype(np.float32)
    O.run_batch(O.FFT, O.COMPLEX_FORWARD, [n], x, batch, 2 * n, False, 1)
    fake_ms = 1.0 + r  # rank 1 is the slower one
    step = bench.max_over_ranks(fake_ms, w, "cpu")
    ok = bool(np.isfinite(x).all())
    bench.dist_finish(w)
    np.save(os.path.join(out, f"rank{r}.npy"), np.array([step, float(ok), w]))


def test_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    from oracle import oracle as O
    O.build()
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        step, ok, w = np.load(tmp_path / f"rank{r}.npy")
        assert step == 2.0 and ok == 1.0 and w == 2  # the max over ranks reached every rank


def test_reference_arm_other_ranks_exit():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--gpus", "2"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
