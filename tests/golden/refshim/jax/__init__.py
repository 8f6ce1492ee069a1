"""Value-only stand-in for jax (test infrastructure; see README.md beside this package)."""
from __future__ import annotations

import numpy as _np

from . import numpy  # noqa: F401
from . import lax  # noqa: F401
from . import scipy  # noqa: F401
from . import tree_util  # noqa: F401
from . import ffi  # noqa: F401
from . import nn  # noqa: F401


class _Config:
    def update(self, *a, **k):
        return None


config = _Config()
Array = _np.ndarray


def jit(f=None, **kw):
    if f is None:
        return lambda g: g
    return f


def vmap(f, in_axes=0, out_axes=0):
    def g(*args):
        n = None
        for a, ax in zip(args, in_axes if isinstance(in_axes, (tuple, list)) else [in_axes] * len(args)):
            if ax is not None:
                n = _np.asarray(a).shape[ax]
                break
        outs = []
        for i in range(n):
            sl = []
            for a, ax in zip(args, in_axes if isinstance(in_axes, (tuple, list)) else [in_axes] * len(args)):
                sl.append(_np.take(_np.asarray(a), i, axis=ax) if ax is not None else a)
            outs.append(_np.asarray(f(*sl)))
        return numpy.asarray(_np.stack(outs, axis=out_axes))
    return g


class custom_vjp:
    def __init__(self, fun, nondiff_argnums=()):
        self.fun = fun

    def defvjp(self, fwd, bwd):
        return None

    def __call__(self, *a, **k):
        return self.fun(*a, **k)


class custom_jvp(custom_vjp):
    def defjvp(self, jvp):
        return jvp


def _no_ad(*a, **k):
    raise NotImplementedError("automatic differentiation is not available in the value-only jax stand-in")


jvp = vjp = linear_transpose = jacfwd = jacrev = value_and_grad = _no_ad

# step of the complex-step derivative: d f(x)/dx_j = Im f(x + i h e_j) / h, exact to rounding for a
# real-analytic f built from operations that extend analytically to complex arguments
COMPLEX_STEP = 1e-30


def grad(f, argnums=0):
    """Gradient of a scalar real-analytic function of one real array by complex steps, one per
    component (what the reference differentiates with it here: the PZ81 XC energy, a sum of
    real-analytic point terms).  Not valid for functions that conjugate or take absolute values."""
    if argnums != 0:
        raise NotImplementedError("grad: argnums != 0")

    def g(x, *rest):
        x = _np.asarray(x, dtype=_np.float64)
        out = _np.empty_like(x)
        flat = out.reshape(-1)
        for j in range(x.size):
            xc = x.astype(_np.complex128).reshape(-1)
            xc[j] += 1j * COMPLEX_STEP
            flat[j] = _np.imag(f(numpy.asarray(xc.reshape(x.shape)), *rest)) / COMPLEX_STEP
        return numpy.asarray(out)
    return g


def pure_callback(f, result_shape, *args, **kw):
    return f(*args)


def devices(*a, **k):
    return []


def block_until_ready(x):
    return x


class ShapeDtypeStruct:
    def __init__(self, shape, dtype):
        self.shape, self.dtype = tuple(shape), dtype
