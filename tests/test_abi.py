"""CPU tests of the C ABI: the library loads and exports every symbol the
header declares; constants agree between header, binding and oracle."""
import os
import re

import pytest

from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "jtgpu.h")


def _header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(jt_[a-z_0-9]+)\s*\(", src)))


def _header_defines():
    out = {}
    for m in re.finditer(r"#define\s+(JT_[A-Z0-9_]+)\s+\(?(-?\d+)\)?", open(HEADER).read()):
        out[m.group(1)] = int(m.group(2))
    return out


@pytest.fixture(scope="module")
def lib():
    from jtransforms_gb300 import build as B
    B.build()
    from jtransforms_gb300 import _native
    return _native.load()


def test_exports_every_declared_symbol(lib):
    import subprocess
    from jtransforms_gb300 import _native
    names = _header_functions()
    assert len(names) >= 15
    syms = subprocess.run(["nm", "-D", "--defined-only", _native.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT\s+(jt_\w+)", syms))
    for n in names:
        assert n in exported, n
        assert hasattr(lib, n)
    # the Python binding declares a signature for each of them
    assert sorted(_native.SIGNATURES) == names


def test_constants_agree(lib):
    from jtransforms_gb300 import _native as N
    from oracle import oracle as O
    d = _header_defines()
    assert d["JT_OK"] == N.OK and d["JT_EBADSIZE"] == N.EBADSIZE and d["JT_ESHORTBUF"] == N.ESHORTBUF
    assert d["JT_ENOTPOW2"] == N.ENOTPOW2 and d["JT_ECUDA"] == N.ECUDA and d["JT_ETIMEOUT"] == N.ETIMEOUT
    for k in ("COMPLEX_FORWARD", "COMPLEX_INVERSE", "REAL_FORWARD", "REAL_FORWARD_FULL", "REAL_INVERSE",
              "REAL_INVERSE_FULL", "FORWARD", "INVERSE"):
        assert d["JT_" + k] == getattr(N, k) == getattr(O, k)
    for k in ("FFT", "DCT", "DST", "DHT"):
        assert d["JT_" + k] == getattr(N, k) == getattr(O, k)


def test_strerror_and_argument_checks(lib):
    import ctypes
    assert lib.jt_strerror(0) == b"ok"
    assert b"power of two" in lib.jt_strerror(-3)
    h = ctypes.c_void_p()
    dims = (ctypes.c_int64 * 3)(0, 0, 0)
    # bad sizes are rejected before any device work
    assert lib.jt_plan_create(0, 1, 1, dims, ctypes.byref(h)) == -1
    dims2 = (ctypes.c_int64 * 3)(1, 8, 0)
    assert lib.jt_plan_create(0, 1, 2, dims2, ctypes.byref(h)) == -1
    assert lib.jt_plan_create(9, 1, 1, dims2, ctypes.byref(h)) == -6
    assert lib.jt_plan_destroy(None) == -6


def test_api_validates_like_reference():
    import jtransforms_gb300 as J
    with pytest.raises(J.IllegalArgumentException):
        J.DoubleFFT_1D(0)
    with pytest.raises(J.IllegalArgumentException):
        J.DoubleFFT_2D(1, 8)
    with pytest.raises(J.IllegalArgumentException):
        J.DoubleFFT_3D(4, 4, 1)
    with pytest.raises(J.IllegalArgumentException):
        J.DoubleDCT_1D(0)
    with pytest.raises(J.IllegalArgumentException):
        J.DoubleDHT_2D(2, 1)


def test_no_silent_cpu_path_without_gpu():
    """Without a GPU the library refuses to run (no fallback)."""
    from tests.conftest import has_gpu
    if has_gpu():
        pytest.skip("GPU present")
    import jtransforms_gb300 as J
    with pytest.raises(J.IllegalStateException):
        J.DoubleFFT_1D(16)


def test_config_setters_are_accepted():
    import jtransforms_gb300 as J
    J.CommonUtils.setThreadsBeginN_1D_FFT_2Threads(1024)
    assert J.CommonUtils.getThreadsBeginN_1D_FFT_2Threads() == 1024
    J.ConcurrencyUtils.setNumberOfThreads(4)
    assert J.ConcurrencyUtils.getNumberOfThreads() == 4
    assert J.CommonUtils.getReminder(10158) == 1693
    assert J.CommonUtils.nextPow2(2 * 10158 - 1) == 32768


def test_split_override_rules(lib):
    """jt_set_split (host logic only): one, two or three passes of at most
    4096 each summing to log2 n, for both precisions; anything else is
    refused and a negative first length clears the override."""
    from jtransforms_gb300 import _native as N
    try:
        assert lib.jt_set_split(N.FLOAT32, 20, 10, 10, 0) == N.OK
        assert lib.jt_set_split(N.FLOAT64, 26, 9, 9, 8) == N.OK       # three passes in double too
        assert lib.jt_set_split(N.FLOAT64, 14, 0, 0, 0) == N.OK
        assert lib.jt_set_split(N.FLOAT32, 20, 10, 9, 0) == N.EINVAL  # sums to 19
        assert lib.jt_set_split(N.FLOAT32, 26, 13, 13, 0) == N.EINVAL  # a pass above 4096
        assert lib.jt_set_split(N.FLOAT64, 24, 13, 6, 5) == N.EINVAL
        assert lib.jt_set_split(2, 20, 10, 10, 0) == N.EINVAL          # no such precision
    finally:
        for prec, lg in ((N.FLOAT32, 20), (N.FLOAT64, 26), (N.FLOAT64, 14)):
            assert lib.jt_set_split(prec, lg, -1, 0, 0) == N.OK
