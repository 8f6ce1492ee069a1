"""jax.numpy on NumPy: FP64 defaults, arrays with the .at[...] update syntax."""
from __future__ import annotations

import numpy as _np


class _At:
    def __init__(self, arr, idx):
        self.arr, self.idx = arr, idx

    def set(self, v, **kw):
        out = _np.array(self.arr, copy=True)
        out[self.idx] = v
        return out.view(JArray)

    def add(self, v, **kw):
        out = _np.array(self.arr, copy=True)
        _np.add.at(out, self.idx, v)
        return out.view(JArray)

    def get(self, **kw):
        return _np.asarray(self.arr)[self.idx].view(JArray)


class _AtIndexer:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _At(self.arr, idx)


class JArray(_np.ndarray):
    @property
    def at(self):
        return _AtIndexer(self)

    def block_until_ready(self):
        return self


def _wrap(x):
    if isinstance(x, _np.ndarray) and not isinstance(x, JArray):
        return x.view(JArray)
    if isinstance(x, tuple):
        return tuple(_wrap(y) for y in x)
    if isinstance(x, list):
        return [_wrap(y) for y in x]
    return x


def _wrapped(f):
    def g(*a, **k):
        k.pop("precision", None)
        return _wrap(f(*a, **k))
    g.__name__ = getattr(f, "__name__", "f")
    return g


def asarray(x, dtype=None):
    return _np.asarray(x, dtype=dtype).view(JArray)


def array(x, dtype=None, copy=True):
    return _np.array(x, dtype=dtype, copy=copy).view(JArray)


ndarray = _np.ndarray
pi = _np.pi
inf = _np.inf
nan = _np.nan
newaxis = None
float64, float32, complex128, complex64 = _np.float64, _np.float32, _np.complex128, _np.complex64
int32, int64, bool_, uint8 = _np.int32, _np.int64, _np.bool_, _np.uint8
dtype = _np.dtype
finfo, iinfo = _np.finfo, _np.iinfo
issubdtype, iscomplexobj = _np.issubdtype, _np.iscomplexobj
complexfloating, floating, integer = _np.complexfloating, _np.floating, _np.integer
ndim, shape, size = _np.ndim, _np.shape, _np.size


def __getattr__(name):
    f = getattr(_np, name)
    return _wrapped(f) if callable(f) else f


class _Sub:
    def __init__(self, mod):
        self._m = mod

    def __getattr__(self, name):
        f = getattr(self._m, name)
        return _wrapped(f) if callable(f) else f


linalg = _Sub(_np.linalg)
fft = _Sub(_np.fft)
