"""Stand-in for ``cupyx.scipy.interpolate`` (golden-fixture generation only)."""
from scipy.interpolate import PchipInterpolator  # noqa: F401
