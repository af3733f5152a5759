"""Stand-in for ``cupyx.scipy.special`` (golden-fixture generation only)."""
from scipy.special import j0, j1  # noqa: F401
