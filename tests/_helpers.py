"""Shared test helpers: the reference tests' RNG and tolerances."""
from __future__ import annotations

import math

import numpy as np

SEED = 20110602  # fft/DoubleFFT_1DTest.java:83


class JavaRandom:
    """java.util.Random: the 48-bit LCG the Java SE specification defines, so
    inputs match the reference tests' `new Random(20110602)`."""

    MULT = 0x5DEECE66D
    MASK = (1 << 48) - 1

    def __init__(self, seed: int):
        self.seed = (seed ^ self.MULT) & self.MASK

    def _next(self, bits: int) -> int:
        self.seed = (self.seed * self.MULT + 0xB) & self.MASK
        r = self.seed >> (48 - bits)
        if r >= 1 << (bits - 1):
            r -= 1 << bits
        return r

    def nextDouble(self) -> float:
        hi = self._next(26) & ((1 << 26) - 1)
        lo = self._next(27) & ((1 << 27) - 1)
        return ((hi << 27) + lo) * (1.0 / (1 << 53))

    def uniform_pm1(self, count: int) -> np.ndarray:
        """count values of 2*nextDouble()-1, the reference tests' inputs."""
        return np.array([2.0 * self.nextDouble() - 1.0 for _ in range(count)])


def rel_l2(got, want) -> float:
    got = np.asarray(got)
    want = np.asarray(want)
    if not np.iscomplexobj(got):
        got = got.astype(np.float64)
    if not np.iscomplexobj(want):
        want = want.astype(np.float64)
    d = np.linalg.norm(got - want)
    nrm = np.linalg.norm(want)
    return float(d / nrm) if nrm > 0 else float(d)


def tol(N: int, dtype) -> float:
    """4 * eps * log2(N) relative L2 (log2 floored at 1 so N <= 2 is not
    held to zero)."""
    eps = float(np.finfo(dtype).eps)
    return 4.0 * eps * max(math.log2(max(N, 2)), 1.0)


def rmse(a, b) -> float:
    """IOUtils.computeRMSE (utils/IOUtils.java:185-197)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2))) if a.size else 0.0
