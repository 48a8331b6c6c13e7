"""Drop-in replacement of jcottaar/seismic ``core/seis_forward2.py``.

``vel_to_seis(vec, vec_diff=None, vec_adjoint=None, adjoint_on_residual=False)``
keeps the reference's signature, shapes, dtypes and assertions
(``core/seis_forward2.py:146-160``) and its outputs
``(result, result_diff, result_adjoint)``:

* ``result``         (nshots*nt*nrec, 1)  seismogram of ``vec``
* ``result_diff``    J @ vec_diff, or None
* ``result_adjoint`` J^T @ vec_adjoint, or J^T @ (result - vec_adjoint) when
  ``adjoint_on_residual``, shape (nz*nx+1, 1), or None

Inputs are FP64 column vectors on the GPU: torch tensors, or any DLPack
array (a CuPy array comes back as CuPy).  The sweeps run in FP32 in the CUDA
engine; outputs are FP64.  The module keeps one engine for the configured
geometry, as the reference keeps its buffers and CUDA graphs in module
globals (``core/seis_forward2.py:13-17,102-176``); like the reference, the
function is not re-entrant across threads.  Unlike the reference it does not
block the host: results are ordered on the current torch stream.

The module-level constants are the reference's (``core/seis_forward2.py:69-101``);
``configure()`` switches to another geometry.
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import Engine
from .geometry import Geometry

# reference constants (core/seis_forward2.py:69-82)
nz = 70
nx = 70
dx = 10
nbc = 120
nt = 999
dt = 1e-3
freq = 15
c1 = -2.5
c2 = 4.0 / 3.0
c3 = -1.0 / 12.0

_geometry = Geometry.reference(nt=nt)
_engine: Engine | None = None


def configure(geometry: Geometry, max_shots_per_chunk: int = 0) -> None:
    """Use another geometry for subsequent vel_to_seis calls (releases the old engine)."""
    global _geometry, _engine
    if _engine is not None:
        _engine.close()
    _geometry = geometry
    _engine = Engine(geometry, max_models=1, max_shots_per_chunk=max_shots_per_chunk)


def geometry() -> Geometry:
    return _geometry


def engine() -> Engine:
    global _engine
    if _engine is None:
        _engine = Engine(_geometry, max_models=1)
    return _engine


def _to_torch(x):
    if x is None:
        return None, None
    if isinstance(x, torch.Tensor):
        return x, None
    mod = type(x).__module__.split(".")[0]
    return torch.from_dlpack(x), mod


def _back(t, mod):
    if t is None or mod is None:
        return t
    if mod == "cupy":
        import cupy  # noqa: F401  (only when the caller passed CuPy arrays)
        return cupy.from_dlpack(t)
    if mod == "numpy":
        return t.cpu().numpy()
    return t


def vel_to_seis(vec, vec_diff=None, vec_adjoint=None, adjoint_on_residual=False):
    g = _geometry
    v, mod = _to_torch(vec)
    vd, _ = _to_torch(vec_diff)
    va, _ = _to_torch(vec_adjoint)
    # input checks of core/seis_forward2.py:153-160
    assert tuple(v.shape) == (g.nv, 1)
    assert va is None or tuple(va.shape) == (g.nrecords, 1)
    assert vd is None or tuple(vd.shape) == (g.nv, 1)
    assert v.dtype == torch.float64
    assert vd is None or vd.dtype == torch.float64
    assert va is None or va.dtype == torch.float64
    eng = engine()
    eng.poll()     # a completed earlier call whose bounded wait gave up raises here
    res, rd, ra, _ = eng.vel_to_seis(v, vd, va, adjoint_on_residual=adjoint_on_residual)
    result = res.reshape(-1, 1)
    result_diff = None if rd is None else rd.reshape(-1, 1)
    result_adjoint = None if ra is None else ra.reshape(-1, 1)
    return _back(result, mod), _back(result_diff, mod), _back(result_adjoint, mod)


def source_wavelet() -> np.ndarray:
    """The Ricker wavelet s of the configured geometry (core/seis_forward2.py:20-45,76-77)."""
    g = _geometry
    nw = int(2.2 / g.freq / g.dt)
    nw = 2 * (nw // 2) + 1
    ncen = nw // 2 + 1
    k = np.arange(1, nw + 1)
    b = ((ncen - k) * g.freq * g.dt * np.pi) ** 2
    w = np.zeros(g.nt)
    w[:nw] = (1.0 - 2.0 * b) * np.exp(-b)
    return w
