"""Autotuner for the pass split of large power-of-two Float32 lengths.

For every length 2^lo .. 2^hi it times complexForward over a device batch of
`--mib` MiB (default 1024, the size class of the headline workload) for each
candidate split:

* one pass (lengths the register kernel holds, up to 2^14);
* two passes 2^a x 2^b (column pass A, transposing row pass B), a, b <= 12;
* three passes 2^a x 2^b x 2^c, each 4..10.

Each candidate is installed with jt_set_split before its plan is created.
Times are CUDA-event medians on the current stream after warm-up, with L2
flushed before every call. The fastest split per length goes into
`jt_plan_table.h`, which the library compiles in. All measurements go to
`plan_table_f32.json` beside it.

    python -m jtransforms_gb300.autotune [--lo 11] [--hi 26] [--mib 1024] [--out-dir DIR]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def candidates(lg: int):
    out = []
    if lg <= 14:
        out.append((0, 0, 0))
    for a in range(max(4, lg - 12), min(12, lg - 4) + 1):
        out.append((a, lg - a, 0))
    if lg >= 14:
        for a in range(4, 11):
            for b in range(4, 11):
                c = lg - a - b
                if 4 <= c <= 10:
                    out.append((a, b, c))
    return out


def time_split(N, J, torch, lg, split, mib, steps, warmup, flush):
    n = 1 << lg
    rc = N.load().jt_set_split(N.FLOAT32, lg, *split)
    if rc != N.OK:
        return None
    try:
        f = J.FloatFFT_1D(n)
    finally:
        N.load().jt_set_split(N.FLOAT32, lg, -1, 0, 0)
    batch = max(1, (mib << 20) // (8 * n))
    x = torch.randn(2 * n * batch, device="cuda", dtype=torch.float32)
    stream = torch.cuda.current_stream()
    times = []
    for s in range(warmup + steps):
        flush()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        f.plan.execute(N.COMPLEX_FORWARD, x, 0, False, batch=batch, dist=2 * n)
        e1.record(stream)
        if s >= warmup:
            times.append((e0, e1))
    torch.cuda.synchronize()
    ms = statistics.median(a.elapsed_time(b) for a, b in times)
    algo = f.plan.algorithm(0)
    del f, x
    return {"ms": ms, "GB/s": 2 * 8 * n * batch / (ms * 1e-3) / 1e9, "batch": batch, "algorithm": algo}


def write_header(best: dict, path: str):
    rows = []
    for lg in range(31):
        s = best.get(lg)
        rows.append("{%d, %d, %d}" % tuple(s) if s is not None else "{-1, -1, -1}")
    none = ", ".join(["{-1, -1, -1}"] * 31)
    body = ",\n    ".join(", ".join(rows[i:i + 8]) for i in range(0, 31, 8))
    with open(path, "w") as fh:
        fh.write("// jt_plan_table.h -- pass split per power-of-two length, indexed by log2 n:\n"
                 "// {0,0,0} one pass, {a,b,0} two passes 2^a (column) x 2^b (row), {a,b,c}\n"
                 "// three passes, {-1,-1,-1} no entry (the engine's rules decide).\n"
                 "// Regenerated by `python -m jtransforms_gb300.autotune` on the target GPU;\n"
                 "// the measurements are in plan_table_f32.json.\n"
                 "#pragma once\n\n"
                 "static const signed char kSplitF32[31][3] = {\n    " + body + ",\n};\n\n"
                 "static const signed char kSplitF64[31][3] = {\n    " + none + ",\n};\n")


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--lo", type=int, default=11)
    ap.add_argument("--hi", type=int, default=26)
    ap.add_argument("--mib", type=int, default=1024)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--out-dir", default="", help="where to write the header and the JSON (default: the package)")
    args = ap.parse_args(argv)
    import torch
    sys.path.insert(0, os.path.dirname(HERE))
    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    if not torch.cuda.is_available():
        print("autotune needs a CUDA device", file=sys.stderr)
        return 2
    flushbuf = torch.empty(64 << 20, dtype=torch.float32, device="cuda")  # 256 MiB > L2

    def flush():
        flushbuf.fill_(1.0)

    results, best = {}, {}
    for lg in range(args.lo, args.hi + 1):
        res = {}
        for sp in candidates(lg):
            r = time_split(N, J, torch, lg, sp, args.mib, args.steps, args.warmup, flush)
            if r is not None:
                res["%d,%d,%d" % sp] = r
        if not res:
            continue
        key = min(res, key=lambda k: res[k]["ms"])
        best[lg] = tuple(int(v) for v in key.split(","))
        results[lg] = {"best": key, "candidates": res}
        print(f"2^{lg}: best {key} {res[key]['GB/s']:.0f} GB/s", flush=True)
    out_dir = args.out_dir or os.path.join(HERE, "csrc")
    os.makedirs(out_dir, exist_ok=True)
    write_header(best, os.path.join(out_dir, "jt_plan_table.h"))
    with open(os.path.join(args.out_dir or HERE, "plan_table_f32.json"), "w") as fh:
        json.dump({"device": torch.cuda.get_device_name(0), "mib_per_call": args.mib, "sizes": results}, fh, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
