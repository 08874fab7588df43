"""ctypes front-end of the CPU oracle (oracle/jt_oracle.cpp).

TEST INFRASTRUCTURE ONLY: tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline leg use this module as the checker.  The product
(``jtransforms_gb300``) never imports it.

The oracle restates JTransforms' algorithms (reference
src/main/java/org/jtransforms/**) on the CPU; ``build()`` compiles it with
``-O2 -ffp-contract=off`` so float and double round like Java.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "jt_oracle.cpp")
LIB = os.path.join(HERE, "libjtoracle.so")

# Operation and kind codes shared with include/jtgpu.h.
COMPLEX_FORWARD, COMPLEX_INVERSE, REAL_FORWARD, REAL_FORWARD_FULL = 0, 1, 2, 3
REAL_INVERSE, REAL_INVERSE_FULL, FORWARD, INVERSE = 4, 5, 6, 7
FFT, DCT, DST, DHT = 0, 1, 2, 3
SPLIT_RADIX, MIXED_RADIX, BLUESTEIN = 0, 1, 2

_lib = None


def build(force: bool = False) -> str:
    """Compiles the oracle into oracle/libjtoracle.so (host compiler, OpenMP)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["g++", "-O2", "-ffp-contract=off", "-fopenmp", "-std=c++17", "-shared",
               "-fPIC", SRC, "-o", LIB + ".tmp"]
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        i64p = ctypes.POINTER(ctypes.c_int64)
        for name, fp in (("jto_run_d", ctypes.c_double), ("jto_run_f", ctypes.c_float)):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, i64p, ctypes.c_void_p, ctypes.c_int]
        for name in ("jto_batch_d", "jto_batch_f"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, i64p, ctypes.c_void_p,
                          ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int]
        L.jto_plan_kind.restype = ctypes.c_int
        L.jto_plan_kind.argtypes = [ctypes.c_int64]
        L.jto_bluestein_size.restype = ctypes.c_int64
        L.jto_bluestein_size.argtypes = [ctypes.c_int64]
        L.jto_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _dims(dims):
    d = (ctypes.c_int64 * 3)(*([int(x) for x in dims] + [0] * (3 - len(dims))))
    return d


def run(kind: int, op: int, dims, a: np.ndarray, scale: bool = False) -> np.ndarray:
    """Runs one transform in place on a contiguous float32/float64 array."""
    assert a.flags.c_contiguous
    if a.dtype == np.float64:
        rc = lib().jto_run_d(kind, op, len(dims), _dims(dims), a.ctypes.data, int(scale))
    elif a.dtype == np.float32:
        rc = lib().jto_run_f(kind, op, len(dims), _dims(dims), a.ctypes.data, int(scale))
    else:
        raise TypeError(a.dtype)
    if rc != 0:
        raise ValueError(f"oracle error {rc} (kind={kind} op={op} dims={dims})")
    return a


def run_batch(kind: int, op: int, dims, a: np.ndarray, batch: int, stride: int,
              scale: bool = False, threads: int = 0) -> np.ndarray:
    """Runs `batch` independent transforms spaced `stride` elements apart,
    one per OpenMP task over `threads` threads (0 = all)."""
    assert a.flags.c_contiguous
    fn = lib().jto_batch_d if a.dtype == np.float64 else lib().jto_batch_f
    rc = fn(kind, op, len(dims), _dims(dims), a.ctypes.data, batch, stride, int(scale), threads)
    if rc != 0:
        raise ValueError(f"oracle error {rc}")
    return a


def plan_kind(n: int) -> int:
    return lib().jto_plan_kind(n)


def bluestein_size(n: int) -> int:
    return lib().jto_bluestein_size(n)


def max_threads() -> int:
    return lib().jto_max_threads()
