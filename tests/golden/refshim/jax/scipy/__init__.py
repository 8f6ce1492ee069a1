from . import special  # noqa: F401
from . import sparse  # noqa: F401
