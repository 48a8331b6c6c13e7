"""Python handle of a ``SeisEngine`` (include/seis_gb300.h) over torch CUDA tensors.

torch supplies device memory and the stream; the sweeps run in the CUDA
library.  There is no other compute path: without a GPU or the library, the
calls raise.
"""
from __future__ import annotations

import ctypes

import torch

from ._lib import SeisError, load
from .geometry import Geometry


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _is_host(x) -> bool:
    return (isinstance(x, torch.Tensor) and x.device.type == "cpu") or type(x).__module__ == "numpy"


def _as_models(x, nv: int, name: str, device, host: bool = False) -> torch.Tensor:
    """(nv,), (nv,1) or (M,nv) FP64 -> contiguous (M, nv) FP64 tensor (no copy when possible):
    on the engine's device, or in host memory for a host call."""
    if not isinstance(x, torch.Tensor):
        x = torch.as_tensor(x) if type(x).__module__ == "numpy" else torch.from_dlpack(x)
    if x.dtype != torch.float64:
        raise TypeError(f"{name} must be float64, got {x.dtype}")
    if host:
        x = x.cpu()
    elif x.device.type != "cuda":
        x = x.to(device)
    if x.dim() == 2 and x.shape[1] == 1 and x.shape[0] == nv:
        x = x.reshape(1, nv)
    elif x.dim() == 1 and x.shape[0] == nv:
        x = x.reshape(1, nv)
    if x.dim() != 2 or x.shape[1] != nv:
        raise ValueError(f"{name} must have shape (nv,), (nv,1) or (M,nv) with nv={nv}, got {tuple(x.shape)}")
    return x.contiguous()


class Engine:
    """One geometry, up to ``max_models`` models per call.

    ``max_shots_per_chunk`` bounds how many shots sweep concurrently (0 = the
    library's default); it sets the workspace size, not the results.
    """

    def __init__(self, geometry: Geometry, max_models: int = 1, max_shots_per_chunk: int = 0, device=None):
        if not torch.cuda.is_available():
            raise RuntimeError("seismic_gb300.Engine needs a CUDA device (no CPU fallback exists)")
        self.lib = load()
        self.geometry = geometry
        self.max_models = int(max_models)
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        self._h = ctypes.c_void_p()
        g, keep = geometry.to_c()
        with torch.cuda.device(self.device):
            torch.cuda.init()
            rc = self.lib.seis_create(ctypes.byref(g), self.max_models, int(max_shots_per_chunk),
                                      ctypes.byref(self._h))
        del keep
        if rc != 0:
            raise SeisError(rc, (self.lib.seis_last_error(None) or b"").decode())

    # ------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.seis_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != 0:
            raise SeisError(rc, (self.lib.seis_last_error(self._h) or b"").decode())

    # ------------------------------------------------------------------
    def vel_to_seis(self, vec, vec_diff=None, vec_adjoint=None, adjoint_on_residual: bool = False,
                    want_misfit: bool = False, stream: torch.cuda.Stream | None = None):
        """Batched vel_to_seis.  Returns (result (M, nrecords), result_diff | None,
        result_adjoint (M, nv) | None, misfit (M,) | None), FP64 on the engine's device.

        vec_adjoint is w (or the target when adjoint_on_residual), shaped (M, nrecords)
        or (nrecords,)/(nrecords,1) for one model.

        Host call: when ``vec`` is in host memory (a CPU tensor or a NumPy array) every
        input is taken from, and every output returned in, host memory (pinned); the
        engine stages the copies itself, overlapping the large ones with the sweeps,
        and the call returns once the outputs are complete, as the reference does."""
        g = self.geometry
        host = _is_host(vec)
        v = _as_models(vec, g.nv, "vec", self.device, host)
        m = v.shape[0]
        if m > self.max_models:
            raise ValueError(f"{m} models exceed the engine's max_models={self.max_models}")
        vd = None if vec_diff is None else _as_models(vec_diff, g.nv, "vec_diff", self.device, host)
        va = None if vec_adjoint is None else _as_models(vec_adjoint, g.nrecords, "vec_adjoint", self.device, host)
        for name, t in (("vec_diff", vd), ("vec_adjoint", va)):
            if t is not None and t.shape[0] != m:
                raise ValueError(f"{name} has {t.shape[0]} models, vec has {m}")
        if want_misfit and va is None:
            raise ValueError("want_misfit needs vec_adjoint")
        opts = dict(dtype=torch.float64, device="cpu", pin_memory=True) if host else \
            dict(dtype=torch.float64, device=self.device)
        res = torch.empty((m, g.nrecords), **opts)
        rd = torch.empty((m, g.nrecords), **opts) if vd is not None else None
        ra = torch.empty((m, g.nv), **opts) if va is not None else None
        mf = torch.empty((m,), **opts) if want_misfit else None
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.device(self.device):
            rc = self.lib.seis_vel_to_seis(self._h, m, _ptr(v), _ptr(vd), _ptr(va), int(bool(adjoint_on_residual)),
                                           _ptr(res), _ptr(rd), _ptr(ra), _ptr(mf), ctypes.c_void_p(st.cuda_stream))
        self._check(rc)
        if host:
            st.synchronize()
            self.poll()
        return res, rd, ra, mf

    def gn_matvec(self, vec, vec_diff, stream: torch.cuda.Stream | None = None):
        """Gauss-Newton product in one engine call: returns (F(vec) (M, nrecords),
        J vec_diff (M, nrecords), J^T J vec_diff (M, nv)); the adjoint is seeded with
        this call's own tangent records (``seis_gn_matvec``)."""
        g = self.geometry
        v = _as_models(vec, g.nv, "vec", self.device)
        m = v.shape[0]
        if m > self.max_models:
            raise ValueError(f"{m} models exceed the engine's max_models={self.max_models}")
        vd = _as_models(vec_diff, g.nv, "vec_diff", self.device)
        if vd.shape[0] != m:
            raise ValueError(f"vec_diff has {vd.shape[0]} models, vec has {m}")
        opts = dict(dtype=torch.float64, device=self.device)
        res = torch.empty((m, g.nrecords), **opts)
        rd = torch.empty((m, g.nrecords), **opts)
        ra = torch.empty((m, g.nv), **opts)
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.device(self.device):
            rc = self.lib.seis_gn_matvec(self._h, m, _ptr(v), _ptr(vd), _ptr(res), _ptr(rd), _ptr(ra),
                                         ctypes.c_void_p(st.cuda_stream))
        self._check(rc)
        return res, rd, ra

    def set_option(self, key: str, value: int) -> None:
        """Engine option, e.g. ``sweep_path``: 0 automatic, 1 tiled per-step sweeps, 2 cluster sweeps,
        3 tiled kernels as one persistent wavefront launch per sweep."""
        self._check(self.lib.seis_set_option(self._h, key.encode(), int(value)))

    def info(self, key: str) -> int:
        v = ctypes.c_int64()
        self._check(self.lib.seis_get_info(self._h, key.encode(), ctypes.byref(v)))
        return int(v.value)

    def check(self) -> None:
        """Wait for the last call and raise if a device-side bounded wait gave up in any
        call since the previous check."""
        self._check(self.lib.seis_device_status(self._h))

    def poll(self) -> None:
        """Raise if a completed call's bounded wait gave up, without synchronising: reads
        the host mirror of the engine's sticky error word, which each call updates in
        stream order at its end.  Meant for callers that have already synchronised (a
        host read of a call's outputs); a failure in a call still running is reported by
        a later poll or by ``check``."""
        if self.info("err_word"):
            self.check()

    @property
    def slots(self) -> int:
        """Shots the engine sweeps concurrently (one chunk)."""
        return int(self.lib.seis_chunk_slots(self._h))

    def stats(self) -> dict:
        """Launch counters and device time (ms) of the last call's sweeps; synchronises the device."""
        torch.cuda.synchronize(self.device)
        launches = ctypes.c_int64()
        fl, al = ctypes.c_int64(), ctypes.c_int64()
        fms, ams = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.seis_stats(self._h, ctypes.byref(launches), ctypes.byref(fms), ctypes.byref(ams),
                                        ctypes.byref(fl), ctypes.byref(al)))
        return {"launches": launches.value, "fwd_ms": fms.value, "adj_ms": ams.value,
                "fwd_step_launches": fl.value, "adj_step_launches": al.value}


def vel_to_seis_multi(engines: list[Engine], vecs: list, vec_adjoints: list | None = None,
                      adjoint_on_residual: bool = False, want_misfit: bool = False,
                      stream: torch.cuda.Stream | None = None):
    """Several engines' batches (models on different geometries) in one forward and one
    reverse wavefront launch (``seis_vel_to_seis_multi``).  ``vecs[i]`` (M_i, nv_i) and
    ``vec_adjoints[i]`` (M_i, nrecords_i) are device FP64 tensors; returns, per engine,
    (result, result_adjoint | None, misfit | None) -- bitwise what each engine's own
    ``vel_to_seis`` returns."""
    n = len(engines)
    if n < 1 or len(vecs) != n or (vec_adjoints is not None and len(vec_adjoints) != n):
        raise ValueError("one vec (and vec_adjoint) per engine")
    if want_misfit and vec_adjoints is None:
        raise ValueError("want_misfit needs vec_adjoints")
    dev = engines[0].device
    vs, vas, res, ras, mfs, nm = [], [], [], [], [], []
    for i, eng in enumerate(engines):
        g = eng.geometry
        v = _as_models(vecs[i], g.nv, "vec", dev)
        m = v.shape[0]
        if m > eng.max_models:
            raise ValueError(f"engine {i}: {m} models exceed max_models={eng.max_models}")
        vs.append(v)
        nm.append(m)
        if vec_adjoints is not None:
            va = _as_models(vec_adjoints[i], g.nrecords, "vec_adjoint", dev)
            if va.shape[0] != m:
                raise ValueError(f"engine {i}: vec_adjoint has {va.shape[0]} models, vec has {m}")
            vas.append(va)
            ras.append(torch.empty((m, g.nv), dtype=torch.float64, device=dev))
        res.append(torch.empty((m, g.nrecords), dtype=torch.float64, device=dev))
        if want_misfit:
            mfs.append(torch.empty((m,), dtype=torch.float64, device=dev))
    arr = lambda ts: (ctypes.c_void_p * n)(*[t.data_ptr() for t in ts])
    hs = (ctypes.c_void_p * n)(*[e._h.value for e in engines])
    st = stream if stream is not None else torch.cuda.current_stream(dev)
    lib = engines[0].lib
    with torch.cuda.device(dev):
        rc = lib.seis_vel_to_seis_multi(n, hs, (ctypes.c_int32 * n)(*nm), arr(vs), arr(vas) if vas else None,
                                        int(bool(adjoint_on_residual)), arr(res), arr(ras) if ras else None,
                                        arr(mfs) if mfs else None, ctypes.c_void_p(st.cuda_stream))
    if rc != 0:
        raise SeisError(rc, (lib.seis_last_error(None) or b"").decode())
    return [(res[i], ras[i] if ras else None, mfs[i] if mfs else None) for i in range(n)]
