"""numpy/scipy stand-in for ``cupyx`` (golden-fixture generation only)."""
