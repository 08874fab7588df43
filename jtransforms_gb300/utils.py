"""Configuration classes of the reference kept for API compatibility.

JTransforms tunes CPU threading through global setters
(utils/CommonUtils.java:47-206, JLargeArrays' ConcurrencyUtils).  On the GPU
they have no effect: the setters are accepted and stored, the getters return
what was set, and nothing in the transform path reads them.
"""
from __future__ import annotations


class CommonUtils:
    _cfg = {"threadsBeginN_1D_FFT_2Threads": 8192, "threadsBeginN_1D_FFT_4Threads": 65536,
            "threadsBeginN_2D": 65536, "threadsBeginN_3D": 65536, "useLargeArrays": False}

    @staticmethod
    def isPowerOf2(x: int) -> bool:
        return x > 0 and (x & (x - 1)) == 0

    @staticmethod
    def nextPow2(x: int) -> int:
        if x < 1:
            raise ValueError("x must be greater or equal 1")
        p = 1
        while p < x:
            p <<= 1
        return p

    @staticmethod
    def getReminder(n: int, factors=(4, 2, 3, 5)) -> int:
        if n <= 0:
            raise ValueError("n must be positive integer")
        r = n
        for f in factors:
            if r == 1:
                break
            while r % f == 0:
                r //= f
        return r


def _add_accessors(cls, key):
    cap = key[0].upper() + key[1:]
    setattr(cls, "set" + cap, staticmethod(lambda v, k=key: cls._cfg.__setitem__(k, v)))
    getter = ("is" if key == "useLargeArrays" else "get") + cap
    setattr(cls, getter, staticmethod(lambda k=key: cls._cfg[k]))


for _k in list(CommonUtils._cfg):
    _add_accessors(CommonUtils, _k)


class ConcurrencyUtils:
    _threads = 1

    @staticmethod
    def setNumberOfThreads(n: int):
        ConcurrencyUtils._threads = max(1, int(n))

    @staticmethod
    def getNumberOfThreads() -> int:
        return ConcurrencyUtils._threads
