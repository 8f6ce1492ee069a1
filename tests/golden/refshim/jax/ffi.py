"""jax.ffi is unavailable: the reference then uses its JAX fallbacks."""


def _unavailable(*a, **k):
    raise RuntimeError("jax.ffi is not available in the value-only jax stand-in")


register_ffi_target = pycapsule = ffi_call = _unavailable
