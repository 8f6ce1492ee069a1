"""jax.nn.sigmoid on NumPy (the numerically stable form)."""
import numpy as _np

from . import numpy as _jnp


def sigmoid(x):
    x = _np.asarray(x)
    if _np.iscomplexobj(x):
        return _jnp.asarray(1.0 / (1.0 + _np.exp(-x)))
    out = _np.where(x >= 0, 1.0 / (1.0 + _np.exp(-_np.abs(x))), _np.exp(-_np.abs(x)) / (1.0 + _np.exp(-_np.abs(x))))
    return _jnp.asarray(out)
