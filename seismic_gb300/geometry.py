"""Acquisition geometry of the FD engine.

Replaces the hard-coded module constants of jcottaar/seismic
``core/seis_forward2.py:69-101`` (70x70 model, dx = 10 m, nbc = 120 absorbing
cells, nt = 999, dt = 1 ms, 15 Hz Ricker, sources at x-cells
{0, 17, 34, 52, 69} one cell below the surface, 70 receivers on the same row)
with a parameterised description.  Positions are converted to padded-grid
indices as ``adjust_sr`` does (``core/seis_forward2.py:60-68``): index =
round(coord/dx) + nbc, and a depth within 0.5 m of the surface moves one row
down.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from ._lib import SeisGeometryC

REFERENCE_SOURCE_CELLS = (0, 17, 34, 52, 69)  # core/seis_forward2.py:88


def _padded_index(coord_m, dx: float, nbc: int, depth: bool) -> np.ndarray:
    coord_m = np.asarray(coord_m, dtype=np.float64)
    idx = (np.round(coord_m / dx) + nbc).astype(np.int64)
    if depth:
        idx = idx + (np.abs(coord_m) < 0.5).astype(np.int64)
    return idx.astype(np.int32)


@dataclass(frozen=True)
class Geometry:
    """Grid, time axis, wavelet and shot/receiver layout of one engine."""
    nz: int = 70
    nx: int = 70
    nbc: int = 120
    nt: int = 999
    dx: float = 10.0
    dt: float = 1e-3
    freq: float = 15.0
    source_x_cells: tuple = REFERENCE_SOURCE_CELLS
    source_z_cell: int = 1
    receiver_x_cells: tuple | None = None   # None: every model column
    receiver_z_cell: int = 1
    src_z: np.ndarray = field(init=False, repr=False, compare=False)
    src_x: np.ndarray = field(init=False, repr=False, compare=False)
    rec_z: np.ndarray = field(init=False, repr=False, compare=False)
    rec_x: np.ndarray = field(init=False, repr=False, compare=False)

    def __post_init__(self):
        if self.nz < 1 or self.nx < 1 or self.nbc < 2 or self.nt < 1:
            raise ValueError("Geometry needs nz, nx >= 1, nbc >= 2, nt >= 1")
        rx = np.arange(self.nx) if self.receiver_x_cells is None else np.asarray(self.receiver_x_cells)
        sx = np.asarray(self.source_x_cells)
        set_ = object.__setattr__
        set_(self, "src_x", _padded_index(sx * self.dx, self.dx, self.nbc, False))
        set_(self, "src_z", _padded_index(np.full(len(sx), self.source_z_cell) * self.dx, self.dx, self.nbc, True))
        set_(self, "rec_x", _padded_index(rx * self.dx, self.dx, self.nbc, False))
        set_(self, "rec_z", _padded_index(np.full(len(rx), self.receiver_z_cell) * self.dx, self.dx, self.nbc,
                                          True))

    # -- constructors ---------------------------------------------------------
    @classmethod
    def reference(cls, nt: int = 999) -> "Geometry":
        """The reference's fixed 70x70 / 5-shot / 70-receiver set-up."""
        return cls(nt=nt)

    @classmethod
    def surface(cls, nz: int, nx: int, nshots: int, nt: int, dx: float = 10.0, dt: float = 1e-3,
                freq: float = 15.0, nbc: int = 120) -> "Geometry":
        """nshots sources spread evenly along the surface row (cells round(linspace(0, nx-1)),
        which for 5 shots on 70 columns gives the reference's {0,17,34,52,69}); a receiver
        on every column."""
        cells = tuple(int(c) for c in np.round(np.linspace(0, nx - 1, nshots)))
        return cls(nz=nz, nx=nx, nbc=nbc, nt=nt, dx=dx, dt=dt, freq=freq, source_x_cells=cells)

    # -- sizes ----------------------------------------------------------------
    @property
    def nshots(self) -> int:
        return int(len(self.src_x))

    @property
    def nrec(self) -> int:
        return int(len(self.rec_x))

    @property
    def nv(self) -> int:
        """Length of a model vector: nz*nx velocities + min_vel."""
        return self.nz * self.nx + 1

    @property
    def nrecords(self) -> int:
        """Length of a record vector: nshots*nt*nrec."""
        return self.nshots * self.nt * self.nrec

    @property
    def padded_shape(self) -> tuple:
        return (self.nz + 2 * self.nbc, self.nx + 2 * self.nbc)

    def cfl(self, vmax: float) -> float:
        return vmax * self.dt / self.dx

    def to_c(self):
        """(SeisGeometryC, keep-alive arrays) for the C ABI."""
        keep = [np.ascontiguousarray(a, dtype=np.int32) for a in (self.src_z, self.src_x, self.rec_z, self.rec_x)]
        ip = ctypes.POINTER(ctypes.c_int32)
        g = SeisGeometryC(self.nz, self.nx, self.nbc, self.nt, float(self.dx), float(self.dt), float(self.freq),
                          self.nshots, keep[0].ctypes.data_as(ip), keep[1].ctypes.data_as(ip), self.nrec,
                          keep[2].ctypes.data_as(ip), keep[3].ctypes.data_as(ip))
        return g, keep
