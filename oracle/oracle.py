"""ctypes front end of the FP64 C oracle (``oracle/fd_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline legs of ``bench.py``, never by the product package.

``OracleGeometry`` restates the reference's geometry set-up
(``core/seis_forward2.py:60-101``: ``adjust_sr`` and the shot/receiver
constants) for any grid; ``vel_to_seis`` mirrors the reference signature
(``core/seis_forward2.py:146``) on NumPy FP64 column vectors.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libfd_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile fd_oracle.c (FP64, no FMA contraction, OpenMP) into _build/."""
    src = os.path.join(_HERE, "fd_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        os.makedirs(_BUILD, exist_ok=True)
        tmp = _LIB_PATH + f".{os.getpid()}.tmp"
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                               src, "-o", tmp, "-lm"])
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


class _Geom(ctypes.Structure):
    _fields_ = [("nz", ctypes.c_int32), ("nx", ctypes.c_int32), ("nbc", ctypes.c_int32),
                ("nt", ctypes.c_int32), ("dx", ctypes.c_double), ("dt", ctypes.c_double),
                ("freq", ctypes.c_double), ("nshots", ctypes.c_int32),
                ("src_z", ctypes.POINTER(ctypes.c_int32)), ("src_x", ctypes.POINTER(ctypes.c_int32)),
                ("nrec", ctypes.c_int32),
                ("rec_z", ctypes.POINTER(ctypes.c_int32)), ("rec_x", ctypes.POINTER(ctypes.c_int32))]


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        dp = ctypes.POINTER(ctypes.c_double)
        _lib.fdo_ricker.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, dp]
        _lib.fdo_ricker.restype = ctypes.c_int
        _lib.fdo_damp.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, dp]
        _lib.fdo_vel_to_seis.argtypes = [ctypes.POINTER(_Geom), dp, dp, dp, ctypes.c_int, dp, dp, dp]
        _lib.fdo_vel_to_seis.restype = ctypes.c_int
        _lib.fdo_batch_vel_to_seis.argtypes = [ctypes.c_int, ctypes.POINTER(_Geom), dp, dp, dp, dp,
                                               ctypes.c_int]
        _lib.fdo_batch_vel_to_seis.restype = ctypes.c_int
        _lib.fdo_set_threads.argtypes = [ctypes.c_int]
    return _lib


def _adjust(coord_m: np.ndarray, dx: float, nbc: int, depth: bool) -> np.ndarray:
    """adjust_sr (core/seis_forward2.py:60-68): metres -> padded index; a depth
    within 0.5 m of the surface moves one row down."""
    coord_m = np.asarray(coord_m, dtype=np.float64)
    idx = (np.round(coord_m / dx) + nbc).astype(np.int64)
    if depth:
        idx = idx + (np.abs(coord_m) < 0.5).astype(np.int64)
    return idx


@dataclass
class OracleGeometry:
    """Padded-grid geometry built the reference's way from model-index positions."""
    nz: int = 70
    nx: int = 70
    nbc: int = 120
    nt: int = 999
    dx: float = 10.0
    dt: float = 1e-3
    freq: float = 15.0
    src_x_cells: tuple = (0, 17, 34, 52, 69)  # core/seis_forward2.py:88
    src_z_cells: int = 1                       # sz = 1*dx (core/seis_forward2.py:90)
    rec_z_cells: int = 1                       # gz = dx (core/seis_forward2.py:92)
    rec_x_cells: tuple | None = None           # default: every model column
    src_z: np.ndarray = field(init=False)
    src_x: np.ndarray = field(init=False)
    rec_z: np.ndarray = field(init=False)
    rec_x: np.ndarray = field(init=False)

    def __post_init__(self):
        rx = np.arange(self.nx) if self.rec_x_cells is None else np.asarray(self.rec_x_cells)
        sx = np.asarray(self.src_x_cells)
        self.src_x = _adjust(sx * self.dx, self.dx, self.nbc, False).astype(np.int32)
        self.src_z = _adjust(np.full(len(sx), self.src_z_cells) * self.dx, self.dx, self.nbc, True).astype(np.int32)
        self.rec_x = _adjust(rx * self.dx, self.dx, self.nbc, False).astype(np.int32)
        self.rec_z = _adjust(np.full(len(rx), self.rec_z_cells) * self.dx, self.dx, self.nbc, True).astype(np.int32)

    @property
    def nshots(self):
        return len(self.src_x)

    @property
    def nrec(self):
        return len(self.rec_x)

    def _c(self):
        keep = [np.ascontiguousarray(a, dtype=np.int32) for a in (self.src_z, self.src_x, self.rec_z, self.rec_x)]
        ip = ctypes.POINTER(ctypes.c_int32)
        g = _Geom(self.nz, self.nx, self.nbc, self.nt, self.dx, self.dt, self.freq, self.nshots,
                  keep[0].ctypes.data_as(ip), keep[1].ctypes.data_as(ip), self.nrec,
                  keep[2].ctypes.data_as(ip), keep[3].ctypes.data_as(ip))
        return g, keep


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def as_geometry(geom) -> OracleGeometry:
    """Accept an OracleGeometry or any object with the same padded-index attributes."""
    if isinstance(geom, OracleGeometry):
        return geom
    og = OracleGeometry(nz=geom.nz, nx=geom.nx, nbc=geom.nbc, nt=geom.nt, dx=geom.dx, dt=geom.dt,
                        freq=geom.freq)
    og.src_z = np.asarray(geom.src_z, np.int32)
    og.src_x = np.asarray(geom.src_x, np.int32)
    og.rec_z = np.asarray(geom.rec_z, np.int32)
    og.rec_x = np.asarray(geom.rec_x, np.int32)
    return og


def ricker(freq: float, dt: float, nt: int) -> np.ndarray:
    w = np.zeros(nt)
    if lib().fdo_ricker(freq, dt, nt, _dp(w)) < 0:
        raise ValueError("nt is smaller than the Ricker wavelet")
    return w


def damp(NZ: int, NX: int, nbc: int, dx: float) -> np.ndarray:
    d = np.zeros((NZ, NX))
    lib().fdo_damp(NZ, NX, nbc, dx, _dp(d))
    return d


def set_threads(n: int) -> None:
    lib().fdo_set_threads(int(n))


def vel_to_seis(geom, vec, vec_diff=None, vec_adjoint=None, adjoint_on_residual=False):
    """FP64 (result, result_diff | None, result_adjoint | None), reference shapes:
    (nshots*nt*nrec, 1), same, (nz*nx+1, 1)."""
    g = as_geometry(geom)
    nv = g.nz * g.nx + 1
    nr = g.nshots * g.nt * g.nrec
    vec = np.ascontiguousarray(np.asarray(vec, np.float64).reshape(-1))
    assert vec.shape == (nv,)
    vd = None if vec_diff is None else np.ascontiguousarray(np.asarray(vec_diff, np.float64).reshape(-1))
    va = None if vec_adjoint is None else np.ascontiguousarray(np.asarray(vec_adjoint, np.float64).reshape(-1))
    assert vd is None or vd.shape == (nv,)
    assert va is None or va.shape == (nr,)
    res = np.zeros(nr)
    rd = np.zeros(nr) if vd is not None else None
    ra = np.zeros(nv) if va is not None else None
    cg, keep = g._c()
    rc = lib().fdo_vel_to_seis(ctypes.byref(cg), _dp(vec), _dp(vd), _dp(va), int(bool(adjoint_on_residual)),
                               _dp(res), _dp(rd), _dp(ra))
    del keep
    if rc != 0:
        raise RuntimeError(f"fdo_vel_to_seis failed with status {rc}")
    return (res[:, None], None if rd is None else rd[:, None], None if ra is None else ra[:, None])


def batch_forward(geom, vecs: np.ndarray, threads: int) -> np.ndarray:
    """Records of many models at once (forward sweeps only), one thread per model."""
    g = as_geometry(geom)
    nv = g.nz * g.nx + 1
    nr = g.nshots * g.nt * g.nrec
    vecs = np.ascontiguousarray(vecs, np.float64).reshape(-1, nv)
    res = np.zeros((vecs.shape[0], nr))
    cg, keep = g._c()
    rc = lib().fdo_batch_vel_to_seis(vecs.shape[0], ctypes.byref(cg), _dp(vecs), None, _dp(res), None, int(threads))
    del keep
    if rc != 0:
        raise RuntimeError(f"fdo_batch_vel_to_seis failed with status {rc}")
    return res


def batch_cost_gradient(geom, vecs: np.ndarray, targets: np.ndarray, threads: int):
    """Records and J^T(F(v)-t) for many models at once, one thread per model."""
    g = as_geometry(geom)
    nv = g.nz * g.nx + 1
    nr = g.nshots * g.nt * g.nrec
    vecs = np.ascontiguousarray(vecs, np.float64).reshape(-1, nv)
    m = vecs.shape[0]
    targets = np.ascontiguousarray(targets, np.float64).reshape(m, nr)
    res = np.zeros((m, nr))
    grads = np.zeros((m, nv))
    cg, keep = g._c()
    rc = lib().fdo_batch_vel_to_seis(m, ctypes.byref(cg), _dp(vecs), _dp(targets), _dp(res), _dp(grads),
                                     int(threads))
    del keep
    if rc != 0:
        raise RuntimeError(f"fdo_batch_vel_to_seis failed with status {rc}")
    return res, grads
