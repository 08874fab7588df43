"""The measured peaks the roofline figures divide by: CUDA-core FMA
throughput (the compute bound of the Double and Float paths) and the read
bandwidth of distributed shared memory within thread-block clusters (the
bound of a plan that exchanges one transform between the CTAs of a
cluster).  The tests check that each measurement runs, returns a positive
figure and orders as the hardware must: FP32 above FP64, a CTA's own shared
memory above its peers'.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def _lib():
    from jtransforms_gb300 import _native as N
    return N, N.load()


def test_fma_peaks_order():
    N, lib = _lib()
    got = {}
    for prec in (N.FLOAT32, N.FLOAT64):
        v = ctypes.c_double()
        assert lib.jt_fma_peak(prec, ctypes.byref(v)) == N.OK
        got[prec] = v.value
    assert got[N.FLOAT64] > 100.0
    assert got[N.FLOAT32] > 10 * got[N.FLOAT64]


@pytest.mark.parametrize("cluster", [2, 16])
def test_dsmem_peak_local_above_remote(cluster):
    N, lib = _lib()
    res = {}
    for remote in (0, 1):
        v, ctas = ctypes.c_double(), ctypes.c_int()
        assert lib.jt_dsmem_peak(cluster, remote, ctypes.byref(v), ctypes.byref(ctas)) == N.OK
        assert ctas.value >= cluster and ctas.value % cluster == 0
        res[remote] = v.value
    assert res[1] > 100.0
    assert res[0] > res[1]


def test_dsmem_peak_rejects_bad_arguments():
    N, lib = _lib()
    v = ctypes.c_double()
    assert lib.jt_dsmem_peak(3, 1, ctypes.byref(v), None) == N.EINVAL
    assert lib.jt_dsmem_peak(32, 1, ctypes.byref(v), None) == N.EINVAL
    assert lib.jt_dsmem_peak(2, 2, ctypes.byref(v), None) == N.EINVAL
    assert lib.jt_dsmem_peak(2, 1, None, None) == N.EINVAL
