"""jax.lax control flow, run eagerly."""
import numpy as _np


def fori_loop(lo, hi, body, init):
    x = init
    for i in range(int(lo), int(hi)):
        x = body(i, x)
    return x


def while_loop(cond, body, init):
    x = init
    while bool(cond(x)):
        x = body(x)
    return x


def cond(pred, tf, ff, *ops):
    return tf(*ops) if bool(pred) else ff(*ops)


def stop_gradient(x):
    return x


def scan(f, init, xs, length=None):
    carry, ys = init, []
    n = length if xs is None else len(xs)
    for i in range(n):
        carry, y = f(carry, None if xs is None else xs[i])
        ys.append(y)
    return carry, _np.stack(ys) if ys and ys[0] is not None else None
