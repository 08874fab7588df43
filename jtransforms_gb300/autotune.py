"""Autotuner for the pass split of large power-of-two lengths, Float32 and
Float64.

For every length 2^lo .. 2^hi it times complexForward over a device batch of
`--mib` MiB (default 1024, the size class of the headline workload) for each
candidate split:

* one pass (lengths the register kernel holds: up to 2^14 for float, 2^13
  for double);
* two passes 2^a x 2^b (column pass A, transposing row pass B), a, b <= 12;
* three passes 2^a x 2^b x 2^c, each 4..10.

Each candidate is installed with jt_set_split before its plan is created.
Times are CUDA-event medians on the current stream after warm-up, with L2
flushed before every call. The fastest split per length and precision goes
into `jt_plan_table.h`, which the library compiles in (a precision that was
not tuned keeps its current table rows). All measurements go to
`plan_table_f32.json` / `plan_table_f64.json` beside it.

With `--tile` it tunes instead the mixed-radix tile kernel: for each size
class ceil(log2 L) and precision it times a 3 * 2^k length (a length the tile
kernel runs) over a 256 MiB batch with each candidate number of elements per
CTA (which sets the lines and threads per CTA), through JT_OPT_TILE_ELEMS,
and writes the fastest into kTileElemsF32 / kTileElemsF64
(`plan_table_tile.json`).

With `--radix` it tunes the tile kernel's pass order: for each size class and
precision it times two lengths of the class, 3 * 2^(k-2) and 7 * 2^(k-3),
over 256 MiB batches with each of the four orders of JT_OPT_RADIX_ORDER
(power-of-two or odd radices first; 16s or 8s for the power of two), and
writes the order with the least summed time into kRadixOrderF32 /
kRadixOrderF64 (`plan_table_radix_<prec>.json`).

    python -m jtransforms_gb300.autotune [--prec f32|f64|both] [--lo 11] [--hi 26] [--mib 1024] [--out-dir DIR]
    python -m jtransforms_gb300.autotune --tile [--prec f32|f64|both] [--out-dir DIR]
    python -m jtransforms_gb300.autotune --radix [--prec f32|f64|both] [--out-dir DIR]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def candidates(lg: int, prec: str = "f32"):
    out = []
    if lg <= (14 if prec == "f32" else 13):
        out.append((0, 0, 0))
    for a in range(max(4, lg - 12), min(12, lg - 4) + 1):
        out.append((a, lg - a, 0))
    # three passes only where two can lose (they measured slower below 2^20
    # for float; double lengths start the search at 2^18)
    if lg >= (14 if prec == "f32" else 18):
        for a in range(4, 11):
            for b in range(4, 11):
                c = lg - a - b
                if 4 <= c <= 10:
                    out.append((a, b, c))
    return out


def time_split(N, J, torch, lg, split, mib, steps, warmup, flush, prec="f32"):
    n = 1 << lg
    P = N.FLOAT32 if prec == "f32" else N.FLOAT64
    esz = 8 if prec == "f32" else 16
    rc = N.load().jt_set_split(P, lg, *split)
    if rc != N.OK:
        return None
    try:
        f = (J.FloatFFT_1D if prec == "f32" else J.DoubleFFT_1D)(n)
    finally:
        N.load().jt_set_split(P, lg, -1, 0, 0)
    batch = max(1, (mib << 20) // (esz * n))
    x = torch.randn(2 * n * batch, device="cuda", dtype=torch.float32 if prec == "f32" else torch.float64)
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
    return {"ms": ms, "GB/s": 2 * esz * n * batch / (ms * 1e-3) / 1e9, "batch": batch, "algorithm": algo}


def read_header(path: str) -> dict:
    """The rows of the current tables: {prec: {lg: split}} for the pass
    splits and {"tile_" + prec: {lg: elements}} for the tile kernel."""
    import re
    out = {"f32": {}, "f64": {}, "tile_f32": {}, "tile_f64": {}, "radix_f32": {}, "radix_f64": {}}
    if not os.path.exists(path):
        return out
    text = open(path).read()
    for prec, name in (("f32", "kSplitF32"), ("f64", "kSplitF64")):
        m = re.search(name + r"\[31\]\[3\] = \{(.*?)\};", text, re.S)
        if not m:
            continue
        rows = re.findall(r"\{(-?\d+), (-?\d+), (-?\d+)\}", m.group(1))
        for lg, r in enumerate(rows):
            if int(r[0]) >= 0:
                out[prec][lg] = tuple(int(v) for v in r)
    for prec, name in (("f32", "kTileElemsF32"), ("f64", "kTileElemsF64")):
        m = re.search(name + r"\[14\] = \{(.*?)\};", text, re.S)
        if m:
            for lg, v in enumerate(int(x) for x in m.group(1).split(",")):
                if v > 0:
                    out["tile_" + prec][lg] = v
    for prec, name in (("f32", "kRadixOrderF32"), ("f64", "kRadixOrderF64")):
        m = re.search(name + r"\[14\] = \{(.*?)\};", text, re.S)
        if m:
            for lg, v in enumerate(int(x) for x in m.group(1).split(",")):
                if v > 0:
                    out["radix_" + prec][lg] = v
    return out


def write_header(best: dict, path: str):
    """best: {prec: {lg: split}, "tile_" + prec: {lg: elements}}."""
    def body(tab):
        rows = ["{%d, %d, %d}" % tuple(tab[lg]) if lg in tab else "{-1, -1, -1}" for lg in range(31)]
        return ",\n    ".join(", ".join(rows[i:i + 8]) for i in range(0, 31, 8))

    def tiles(tab):
        return ", ".join(str(tab.get(lg, 0)) for lg in range(14))
    with open(path, "w") as fh:
        fh.write("// jt_plan_table.h -- pass split per power-of-two length, indexed by log2 n:\n"
                 "// {0,0,0} one pass, {a,b,0} two passes 2^a (column) x 2^b (row), {a,b,c}\n"
                 "// three passes, {-1,-1,-1} no entry (the engine's rules decide).\n"
                 "// Regenerated by `python -m jtransforms_gb300.autotune` on the target GPU;\n"
                 "// the measurements are in plan_table_f32.json and plan_table_f64.json.\n"
                 "#pragma once\n\n"
                 "static const signed char kSplitF32[31][3] = {\n    " + body(best["f32"]) + ",\n};\n\n"
                 "static const signed char kSplitF64[31][3] = {\n    " + body(best["f64"]) + ",\n};\n\n"
                 "// Elements per CTA of the generic tile kernel (mixed-radix lengths), indexed\n"
                 "// by ceil(log2 L); 0: the default (4096 float, 2048 double).\n"
                 "static const short kTileElemsF32[14] = {" + tiles(best.get("tile_f32", {})) + "};\n"
                 "static const short kTileElemsF64[14] = {" + tiles(best.get("tile_f64", {})) + "};\n\n"
                 "// Pass order of the generic tile kernel (direct_radices' `order`), indexed by\n"
                 "// ceil(log2 L); 0: power-of-two radices (16s) first.\n"
                 "static const signed char kRadixOrderF32[14] = {" + tiles(best.get("radix_f32", {})) + "};\n"
                 "static const signed char kRadixOrderF64[14] = {" + tiles(best.get("radix_f64", {})) + "};\n")


def time_tile(N, J, torch, n, elems, prec, flush, steps=5, warmup=3):
    P = N.FLOAT32 if prec == "f32" else N.FLOAT64
    esz = 8 if prec == "f32" else 16
    prev = N.set_option(N.OPT_TILE_ELEMS, elems) if elems else None
    try:
        f = (J.FloatFFT_1D if prec == "f32" else J.DoubleFFT_1D)(n)
        batch = max(1, (256 << 20) // (esz * n))
        x = torch.randn(2 * n * batch, device="cuda", dtype=torch.float32 if prec == "f32" else torch.float64)
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
        assert f.plan.algorithm(0) == 0  # one tile pass
        return {"ms": ms, "GB/s": 2 * esz * n * batch / (ms * 1e-3) / 1e9, "batch": batch}
    finally:
        if elems:
            N.set_option(N.OPT_TILE_ELEMS, prev)


def time_radix(N, J, torch, n, order, prec, flush, steps=5, warmup=3):
    prev = N.set_option(N.OPT_RADIX_ORDER, order)
    try:
        return time_tile(N, J, torch, n, 0, prec, flush, steps, warmup)
    finally:
        N.set_option(N.OPT_RADIX_ORDER, prev)


def tune_radix(N, J, torch, precs, flush, out_dir):
    best = {}
    for prec in precs:
        res, tab = {}, {}
        for lg in range(4, 14 if prec == "f32" else 13):
            lengths = [3 << (lg - 2), 7 << (lg - 3)]  # both with ceil(log2 n) = lg
            cand = {}
            for order in range(4):
                cand[str(order)] = {str(n): time_radix(N, J, torch, n, order, prec, flush) for n in lengths}
            total = {k: sum(v["ms"] for v in c.values()) for k, c in cand.items()}
            key = min(total, key=total.get)
            tab[lg] = int(key)
            res[lg] = {"lengths": lengths, "best": int(key), "summed_ms": total, "candidates": cand}
            print(f"radix order {prec} class 2^{lg} {lengths}: best {key} "
                  f"({total[key]:.3f} ms against {total['0']:.3f} ms for order 0)", flush=True)
        best["radix_" + prec] = tab
        with open(os.path.join(out_dir, f"plan_table_radix_{prec}.json"), "w") as fh:
            json.dump({"device": torch.cuda.get_device_name(0), "mib_per_call": 256, "sizes": res}, fh, indent=1)
    return best


def tune_tiles(N, J, torch, precs, flush, out_dir):
    best = {}
    for prec in precs:
        res, tab = {}, {}
        for lg in range(4, 14 if prec == "f32" else 13):
            n = 3 << (lg - 2)  # in (2^(lg-1), 2^lg]: ceil(log2 n) = lg
            cand = {}
            for elems in (512, 1024, 2048, 4096, 8192, 16384):
                if elems < n:
                    continue
                cand[str(elems)] = time_tile(N, J, torch, n, elems, prec, flush)
            key = min(cand, key=lambda k: cand[k]["ms"])
            tab[lg] = int(key)
            res[lg] = {"n": n, "best": int(key), "candidates": cand}
            print(f"tile {prec} n={n}: best {key} elements per CTA, {cand[key]['GB/s']:.0f} GB/s", flush=True)
        best["tile_" + prec] = tab
        with open(os.path.join(out_dir, f"plan_table_tile_{prec}.json"), "w") as fh:
            json.dump({"device": torch.cuda.get_device_name(0), "mib_per_call": 256, "sizes": res}, fh, indent=1)
    return best


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--prec", choices=["f32", "f64", "both"], default="both")
    ap.add_argument("--lo", type=int, default=11)
    ap.add_argument("--hi", type=int, default=26)
    ap.add_argument("--mib", type=int, default=1024)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--out-dir", default="", help="where to write the header and the JSON (default: the package)")
    ap.add_argument("--tile", action="store_true", help="tune the mixed-radix tile kernel's elements per CTA")
    ap.add_argument("--radix", action="store_true", help="tune the mixed-radix tile kernel's pass order")
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

    out_dir = args.out_dir or os.path.join(HERE, "csrc")
    os.makedirs(out_dir, exist_ok=True)
    header = os.path.join(out_dir, "jt_plan_table.h")
    best = read_header(os.path.join(HERE, "csrc", "jt_plan_table.h"))
    precs = ["f32", "f64"] if args.prec == "both" else [args.prec]
    if args.tile:
        best.update(tune_tiles(N, J, torch, precs, flush, args.out_dir or HERE))
        write_header(best, header)
        return 0
    if args.radix:
        best.update(tune_radix(N, J, torch, precs, flush, args.out_dir or HERE))
        write_header(best, header)
        return 0
    for prec in precs:
        results = {}
        best[prec] = {}
        for lg in range(args.lo, args.hi + 1):
            res = {}
            for sp in candidates(lg, prec):
                try:
                    r = time_split(N, J, torch, lg, sp, args.mib, args.steps, args.warmup, flush, prec)
                except (N.IllegalArgumentException, N.IllegalStateException) as e:
                    print(f"{prec} 2^{lg} {sp}: skipped ({e})", flush=True)
                    r = None
                if r is not None:
                    res["%d,%d,%d" % sp] = r
            if not res:
                continue
            key = min(res, key=lambda k: res[k]["ms"])
            best[prec][lg] = tuple(int(v) for v in key.split(","))
            results[lg] = {"best": key, "candidates": res}
            print(f"{prec} 2^{lg}: best {key} {res[key]['GB/s']:.0f} GB/s", flush=True)
        with open(os.path.join(args.out_dir or HERE, f"plan_table_{prec}.json"), "w") as fh:
            json.dump({"device": torch.cuda.get_device_name(0), "mib_per_call": args.mib, "sizes": results}, fh,
                      indent=1)
    write_header(best, header)
    return 0


if __name__ == "__main__":
    sys.exit(main())
