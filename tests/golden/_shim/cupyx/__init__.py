"""``cupyx`` stand-in for the golden-vector shim: maps to SciPy on the host."""
from . import scipy  # noqa: F401
