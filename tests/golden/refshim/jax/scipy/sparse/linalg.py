def bicgstab(*a, **k):
    raise NotImplementedError("bicgstab needs jax transforms; not available in the value-only stand-in")
