"""ctypes binding of libjtgpu.so (include/jtgpu.h).

The library is the only compute path: if it cannot be loaded, every transform
raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libjtgpu.so")

# status codes
OK, EBADSIZE, ESHORTBUF, ENOTPOW2, ECUDA, ETIMEOUT, EINVAL, ENOMEM, ENODEV, ETOOBIG = 0, -1, -2, -3, -4, -5, -6, -7, -8, -9
ESCRATCH = -10
# kinds / precisions / ops
FFT, DCT, DST, DHT = 0, 1, 2, 3
FLOAT32, FLOAT64 = 0, 1
COMPLEX_FORWARD, COMPLEX_INVERSE, REAL_FORWARD, REAL_FORWARD_FULL = 0, 1, 2, 3
REAL_INVERSE, REAL_INVERSE_FULL, FORWARD, INVERSE = 4, 5, 6, 7
MODE_FP32, MODE_TC_SPLIT = 0, 1

# Every function include/jtgpu.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_int64
SIGNATURES = {
    "jt_plan_create": (_I, [_I, _I, _I, ctypes.POINTER(_L), ctypes.POINTER(_P)]),
    "jt_plan_destroy": (_I, [_P]),
    "jt_plan_extent": (_I, [_P, _I, ctypes.POINTER(_L)]),
    "jt_plan_set_mode": (_I, [_P, _I]),
    "jt_set_split": (_I, [_I, _I, _I, _I, _I]),
    "jt_execute": (_I, [_P, _I, _P, _L, _L, _I]),
    "jt_execute_batch": (_I, [_P, _I, _P, _L, _L, _L, _L, _I]),
    "jt_execute_device": (_I, [_P, _I, _P, _L, _L, _I, _P]),
    "jt_synchronize": (_I, []),
    "jt_check_error": (_I, []),
    "jt_batch_create": (_I, [_I, ctypes.POINTER(_P), ctypes.POINTER(_I), ctypes.POINTER(_P), ctypes.POINTER(_I), ctypes.POINTER(_P)]),
    "jt_batch_run": (_I, [_P, _P]),
    "jt_batch_run_per_transform": (_I, [_P, _P]),
    "jt_batch_run_graph": (_I, [_P, _P]),
    "jt_batch_destroy": (_I, [_P]),
    "jt_strerror": (ctypes.c_char_p, [_I]),
    "jt_last_cuda_error": (_I, []),
    "jt_launch_count": (_L, [_I]),
    "jt_plan_algorithm": (_I, [_P, _I]),
    "jt_set_option": (_I, [_I, _I]),
    "jt_execute_device_noalloc": (_I, [_P, _I, _P, _P, _L, _I, _P]),
    "jt_fma_peak": (_I, [_I, ctypes.POINTER(ctypes.c_double)]),
    "jt_dsmem_peak": (_I, [_I, _I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_I)]),
}
OPT_TMA_PIPELINE, OPT_DIRECT_MAX_F32, OPT_DIRECT_MAX_F64, OPT_COLUMN_KERNEL, OPT_TWOPASS_CHUNK_MB = 0, 1, 2, 3, 4
OPT_THREEPASS_MIN_LOG2, OPT_HOST_PIECE_MB = 5, 6
OPT_ARENA_LIMIT_MB, OPT_BATCH_WAIT_POLLS, OPT_BATCH_STALL_TEST = 7, 8, 9
OPT_TILE_ELEMS, OPT_REAL_FUSED_F32, OPT_RADIX_ORDER = 10, 11, 12

_lib = None
_lock = threading.Lock()


class IllegalArgumentException(ValueError):
    """Java's IllegalArgumentException (bad sizes, non-power-of-two 2D/3D real transforms)."""


class ArrayIndexOutOfBoundsException(IndexError):
    """Java's ArrayIndexOutOfBoundsException (array shorter than offset + extent)."""


class IllegalStateException(RuntimeError):
    """Device-side failure (CUDA error, out of memory, timed-out wait, no GPU)."""


def load(build_if_missing: bool = True):
    """Loads libjtgpu.so, building it in-tree with nvcc if it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH) and build_if_missing:
            from . import build as _b
            _b.build()
        if not os.path.exists(LIB_PATH):
            raise IllegalStateException("libjtgpu.so is not built; run jtransforms_gb300.build.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
        return L


def strerror(code: int) -> str:
    return load().jt_strerror(code).decode()


def check(code: int, what: str = ""):
    if code == OK:
        return
    msg = strerror(code)
    if what:
        msg = f"{what}: {msg}"
    if code in (EBADSIZE, ENOTPOW2):
        raise IllegalArgumentException(msg)
    if code == ESHORTBUF:
        raise ArrayIndexOutOfBoundsException(msg)
    if code in (EINVAL, ETOOBIG, ESCRATCH):
        raise IllegalArgumentException(msg)
    cu = load().jt_last_cuda_error()
    raise IllegalStateException(f"{msg} (cuda error {cu})")


class Plan:
    """Owns one jt_plan handle; released when the object is collected."""

    def __init__(self, kind: int, prec: int, dims):
        self._lib = load()
        d = (ctypes.c_int64 * 3)(*(list(int(x) for x in dims) + [0] * (3 - len(dims))))
        h = ctypes.c_void_p()
        check(self._lib.jt_plan_create(kind, prec, len(dims), d, ctypes.byref(h)))
        self.handle = h
        self.kind, self.prec, self.dims = kind, prec, tuple(int(x) for x in dims)
        self.dtype = np.float32 if prec == FLOAT32 else np.float64

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self._lib.jt_plan_destroy(h)
            except Exception:
                pass
            self.handle = None

    def extent(self, op: int) -> int:
        v = ctypes.c_int64()
        check(self._lib.jt_plan_extent(self.handle, op, ctypes.byref(v)))
        return v.value

    def set_mode(self, mode: int):
        check(self._lib.jt_plan_set_mode(self.handle, mode))

    def algorithm(self, axis: int = 0) -> int:
        return self._lib.jt_plan_algorithm(self.handle, axis)

    def execute(self, op: int, a, offa: int = 0, scale: bool = False, batch: int = 1, dist: int = 0):
        """Runs op in place on `a`: a host numpy array (copied to the GPU and
        back) or a CUDA tensor (run on the current torch stream)."""
        if isinstance(a, np.ndarray):
            if a.dtype != self.dtype:
                raise TypeError(f"array dtype {a.dtype} does not match the transform's {np.dtype(self.dtype)}")
            if not (a.flags.c_contiguous and a.flags.writeable):
                raise IllegalArgumentException("array must be C-contiguous and writeable")
            n = a.size
            if batch == 1:
                rc = self._lib.jt_execute(self.handle, op, a.ctypes.data, n, int(offa), int(bool(scale)))
            else:
                rc = self._lib.jt_execute_batch(self.handle, op, a.ctypes.data, n, int(offa), int(batch), int(dist),
                                                int(bool(scale)))
            check(rc)
            return a
        # torch tensor on the GPU
        try:
            import torch
        except ImportError as e:  # pragma: no cover
            raise TypeError("expected a numpy array or a CUDA tensor") from e
        if not (isinstance(a, torch.Tensor) and a.is_cuda):
            raise TypeError("expected a numpy array or a CUDA tensor")
        want = torch.float32 if self.prec == FLOAT32 else torch.float64
        if a.dtype != want or not a.is_contiguous():
            raise TypeError("CUDA tensor must be contiguous with the transform's dtype")
        ext = self.extent(op)
        if int(offa) < 0 or int(offa) + (batch - 1) * max(dist, ext) + ext > a.numel():
            raise ArrayIndexOutOfBoundsException("tensor too short for offset and transform extent")
        ptr = a.data_ptr() + int(offa) * a.element_size()
        stream = torch.cuda.current_stream(a.device).cuda_stream
        check(self._lib.jt_execute_device(self.handle, op, ctypes.c_void_p(ptr), int(batch),
                                          int(dist if batch > 1 else ext + (ext & 1)), int(bool(scale)),
                                          ctypes.c_void_p(stream)))
        return a


def set_option(option: int, value: int) -> int:
    """Sets a global library option (OPT_*); returns the previous value."""
    return load().jt_set_option(option, value)


def launch_count(reset: bool = False) -> int:
    return load().jt_launch_count(int(reset))


class Batch:
    """Many 1D transforms of different plans run as one persistent launch
    (jt_batch_create / jt_batch_run / jt_batch_run_graph).

    `items` is a list of (Plan, op, tensor_or_device_ptr, scale).  Arrays
    are device memory; the batch records their addresses, so they must stay
    alive and in place while the batch is used."""

    def __init__(self, items):
        self._lib = load()
        self._keep = items
        n = len(items)
        plans = (ctypes.c_void_p * n)(*[it[0].handle.value for it in items])
        ops = (ctypes.c_int * n)(*[int(it[1]) for it in items])
        ptrs = (ctypes.c_void_p * n)(*[(it[2].data_ptr() if hasattr(it[2], "data_ptr") else int(it[2])) for it in items])
        scales = (ctypes.c_int * n)(*[int(bool(it[3])) for it in items])
        h = ctypes.c_void_p()
        check(self._lib.jt_batch_create(n, plans, ops, ptrs, scales, ctypes.byref(h)))
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self._lib.jt_batch_destroy(h)
            except Exception:
                pass
            self.handle = None

    @staticmethod
    def _stream(stream):
        if stream is None:
            import torch
            return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        return ctypes.c_void_p(int(stream))

    def run(self, stream=None):
        """One persistent launch (asynchronous)."""
        check(self._lib.jt_batch_run(self.handle, self._stream(stream)))

    def run_graph(self, stream=None):
        """The same launch captured once into a CUDA graph, then replayed."""
        check(self._lib.jt_batch_run_graph(self.handle, self._stream(stream)))

    def run_per_transform(self, stream=None):
        """The baseline: each transform's own launches, one after another."""
        check(self._lib.jt_batch_run_per_transform(self.handle, self._stream(stream)))
