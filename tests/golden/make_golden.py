"""Regenerates tests/golden/fftw_golden.npz from JTransforms' own test
resources (src/test/resources/fftw{n}.in/.out: raw little-endian complex128,
forward DFT computed by FFTW, read by fft/DoubleFFT_1DTest.java:156-206).

Run with the reference checkout as argument 1, or in JTRANSFORMS_REFERENCE.
Sizes up to 10158 are stored (they cover every plan of the reference:
power of two, mixed radix with radices 3, 5, 7, 11, 13 and 31, and Bluestein
at 10158 = 2*3*1693); the larger files are only read when the reference is
present (tests/test_oracle.py).
"""
import os
import sys

import numpy as np

MAX_N = 10158


def main(root):
    res = os.path.join(root, "src", "test", "resources")
    sizes = [int(s) for s in open(os.path.join(res, "sizes.txt")).read().split()]
    out = {"sizes": np.array([n for n in sizes if n <= MAX_N], dtype=np.int64)}
    for n in sizes:
        if n > MAX_N:
            continue
        out[f"in{n}"] = np.fromfile(os.path.join(res, f"fftw{n}.in"), "<f8")
        out[f"out{n}"] = np.fromfile(os.path.join(res, f"fftw{n}.out"), "<f8")
        assert out[f"in{n}"].size == 2 * n and out[f"out{n}"].size == 2 * n
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fftw_golden.npz")
    np.savez(dst, **out)
    print(dst, sum(v.nbytes for v in out.values()))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("JTRANSFORMS_REFERENCE")
    if not root:
        sys.exit("usage: make_golden.py <JTransforms checkout> (or set JTRANSFORMS_REFERENCE)")
    main(root)
