"""seismic_gb300 -- GB300-native (sm_103a) 2-D acoustic finite-difference engine.

A from-scratch engine for the forward, tangent (J v) and adjoint (J^T w)
sweeps of jcottaar/seismic's ``core/seis_forward2.py``, with the reference's
``vel_to_seis`` call signature (``seismic_gb300.seis_forward2``).

Submodules:
  geometry      acquisition geometry (grid, wavelet, shots, receivers)
  engine        Engine: batched sweeps through the C ABI (include/seis_gb300.h)
  seis_forward2 drop-in ``vel_to_seis``
  synthetic     seeded velocity models (layered / faulted / curved)
"""
from .geometry import Geometry  # noqa: F401


def build(force: bool = False) -> str:
    """Compile the CUDA library for sm_103a (in-tree, ``seismic_gb300/_build``)."""
    from ._lib import build as _build
    return _build(force=force)
