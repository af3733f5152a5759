"""Stand-in for ``cupyx.scipy``: ``special`` and ``interpolate`` map to scipy."""
from . import special, interpolate  # noqa: F401
