"""DCT / DST / DHT classes with JTransforms' Java API
(org.jtransforms.dct, .dst, .dht).

    forward(a, scale) / forward(a, offa, scale)      DCT-II / DST-II
    inverse(a, scale) / inverse(a, offa, scale)      DCT-III / DST-III
    DHT: forward(a) / forward(a, offa); inverse(a, scale) / inverse(a, offa, scale)

scale=True gives the orthonormal transforms (dct/DoubleDCT_1D.java:191-193).
Unscaled outputs follow the reference exactly, including its different
normalisation for power-of-two and other sizes.

Reference: dct/DoubleDCT_1D.java:84-440, dct/DoubleDCT_2D.java,
dct/DoubleDCT_3D.java, dst/DoubleDST_1D.java:55-328, dst/DoubleDST_2D.java,
dst/DoubleDST_3D.java, dht/DoubleDHT_1D.java:55-276, dht/DoubleDHT_2D.java,
dht/DoubleDHT_3D.java and the Float* twins.
"""
from __future__ import annotations

from . import _arrays
from . import _native as N
from ._native import IllegalArgumentException


def _off_scale(args, name):
    if len(args) == 1:
        return 0, bool(args[0])
    if len(args) == 2:
        return int(args[0]), bool(args[1])
    raise TypeError(f"{name}(a, [offa,] scale)")


class _R2RBase:
    _prec = N.FLOAT64
    _kind = N.DCT
    _nd = 1

    def __init__(self, *dims):
        if len(dims) == 1:
            if dims[0] < 1:
                raise IllegalArgumentException("n must be greater than 0")
        else:
            names = {2: "rows and columns", 3: "slices, rows and columns"}[len(dims)]
            if any(d <= 1 for d in dims):
                raise IllegalArgumentException(f"{names} must be greater than 1")
        self._plan = N.Plan(self._kind, self._prec, dims)

    def _run(self, op, a, offa, scale):
        return _arrays.run(self._plan, op, a, offa, scale)

    @property
    def plan(self) -> N.Plan:
        return self._plan


class _CosSin(_R2RBase):
    def forward(self, a, *args):
        offa, scale = _off_scale(args, "forward")
        self._run(N.FORWARD, a, offa, scale)

    def inverse(self, a, *args):
        offa, scale = _off_scale(args, "inverse")
        self._run(N.INVERSE, a, offa, scale)


class _Hartley(_R2RBase):
    _kind = N.DHT

    def forward(self, a, offa: int = 0):
        self._run(N.FORWARD, a, offa, False)

    def inverse(self, a, *args):
        offa, scale = _off_scale(args, "inverse")
        self._run(N.INVERSE, a, offa, scale)


def _make(name, base, kind, prec, nd, doc):
    def __init__(self, *dims):
        if len(dims) != nd:
            raise TypeError(f"{name} takes {nd} size argument(s)")
        _R2RBase.__init__(self, *dims)
    return type(name, (base,), {"__init__": __init__, "_kind": kind, "_prec": prec, "_nd": nd, "__doc__": doc})


_classes = {}
for _kname, _kind, _base, _pkg in (("DCT", N.DCT, _CosSin, "dct"), ("DST", N.DST, _CosSin, "dst"), ("DHT", N.DHT, _Hartley, "dht")):
    for _pname, _prec in (("Double", N.FLOAT64), ("Float", N.FLOAT32)):
        for _nd in (1, 2, 3):
            _n = f"{_pname}{_kname}_{_nd}D"
            _classes[_n] = _make(_n, _base, _kind, _prec, _nd, f"{_pkg}/{_n}.java counterpart.")

DoubleDCT_1D = _classes["DoubleDCT_1D"]
DoubleDCT_2D = _classes["DoubleDCT_2D"]
DoubleDCT_3D = _classes["DoubleDCT_3D"]
FloatDCT_1D = _classes["FloatDCT_1D"]
FloatDCT_2D = _classes["FloatDCT_2D"]
FloatDCT_3D = _classes["FloatDCT_3D"]
DoubleDST_1D = _classes["DoubleDST_1D"]
DoubleDST_2D = _classes["DoubleDST_2D"]
DoubleDST_3D = _classes["DoubleDST_3D"]
FloatDST_1D = _classes["FloatDST_1D"]
FloatDST_2D = _classes["FloatDST_2D"]
FloatDST_3D = _classes["FloatDST_3D"]
DoubleDHT_1D = _classes["DoubleDHT_1D"]
DoubleDHT_2D = _classes["DoubleDHT_2D"]
DoubleDHT_3D = _classes["DoubleDHT_3D"]
FloatDHT_1D = _classes["FloatDHT_1D"]
FloatDHT_2D = _classes["FloatDHT_2D"]
FloatDHT_3D = _classes["FloatDHT_3D"]
