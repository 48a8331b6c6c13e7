"""Build and load the engine's shared library (``_build/libseis_gb300.so``).

The library is the C ABI declared in ``include/seis_gb300.h``.  It is built
in-tree with nvcc for sm_103a only; importing the compute path without it
raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

_PKG = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_PKG)
CSRC = os.path.join(_PKG, "csrc")
BUILD_DIR = os.path.join(_PKG, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libseis_gb300.so")
INCLUDE_DIR = os.path.join(_ROOT, "include")

# translation units of the library; compiled in parallel, linked once
SOURCES = ["engine.cu", "noalloc.cu", "optim.cu"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-I" + INCLUDE_DIR]

_lock = threading.Lock()
_lib = None


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE_DIR, "seis_gb300.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every translation unit for sm_103a and link libseis_gb300.so."""
    with _lock:
        if not force and not _stale():
            return LIB_PATH
        os.makedirs(BUILD_DIR, exist_ok=True)
        nvcc = _nvcc()
        objs, procs = [], []
        for src in SOURCES:
            obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
            cmd = [nvcc, *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
            if verbose:
                print(" ".join(cmd))
            procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), cmd))
            objs.append(obj)
        for p, cmd in procs:
            out, _ = p.communicate()
            if p.returncode != 0:
                raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{out.decode(errors='replace')}")
        tmp = LIB_PATH + f".{os.getpid()}.tmp"
        # static cudart: the library needs no CUDA runtime on the loader path
        subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-cudart", "static",
                               *objs, "-o", tmp])
        os.replace(tmp, LIB_PATH)
        return LIB_PATH


class SeisGeometryC(ctypes.Structure):
    """ctypes mirror of ``SeisGeometry`` (include/seis_gb300.h)."""
    _fields_ = [("nz", ctypes.c_int32), ("nx", ctypes.c_int32), ("nbc", ctypes.c_int32),
                ("nt", ctypes.c_int32), ("dx", ctypes.c_double), ("dt", ctypes.c_double),
                ("freq", ctypes.c_double), ("nshots", ctypes.c_int32),
                ("src_z", ctypes.POINTER(ctypes.c_int32)), ("src_x", ctypes.POINTER(ctypes.c_int32)),
                ("nrec", ctypes.c_int32),
                ("rec_z", ctypes.POINTER(ctypes.c_int32)), ("rec_x", ctypes.POINTER(ctypes.c_int32))]


# name -> (restype, argtypes) of every symbol the header declares
_VP = ctypes.c_void_p
EXPORTS = {
    "seis_create": (ctypes.c_int, [ctypes.POINTER(SeisGeometryC), ctypes.c_int32, ctypes.c_int32,
                                   ctypes.POINTER(_VP)]),
    "seis_destroy": (ctypes.c_int, [_VP]),
    "seis_last_error": (ctypes.c_char_p, [_VP]),
    "seis_vel_to_seis": (ctypes.c_int, [_VP, ctypes.c_int32, _VP, _VP, _VP, ctypes.c_int32, _VP, _VP, _VP, _VP,
                                        _VP]),
    "seis_gn_matvec": (ctypes.c_int, [_VP, ctypes.c_int32, _VP, _VP, _VP, _VP, _VP, _VP]),
    "seis_vel_to_seis_multi": (ctypes.c_int, [ctypes.c_int32, _VP, _VP, _VP, _VP, ctypes.c_int32, _VP, _VP, _VP,
                                              _VP]),
    "seis_chunk_slots": (ctypes.c_int, [_VP]),
    "seis_set_option": (ctypes.c_int, [_VP, ctypes.c_char_p, ctypes.c_int64]),
    "seis_get_info": (ctypes.c_int, [_VP, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64)]),
    "seis_device_status": (ctypes.c_int, [_VP]),
    "seis_tv_prior": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                     ctypes.c_double, _VP, _VP, _VP, _VP]),
    "seis_lbfgs_direction": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32] + [_VP] * 9),
    "seis_reduce": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _VP, _VP, _VP, _VP]),
    "seis_lbfgs_state_bytes": (ctypes.c_int64, [ctypes.c_int32, ctypes.c_int32]),
    "seis_lbfgs_step": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                       ctypes.c_double] + [_VP] * 7),
    "seis_forward_noalloc": (ctypes.c_int, [ctypes.POINTER(SeisGeometryC), _VP, _VP, _VP]),
    "seis_stats": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64),
                                  ctypes.POINTER(ctypes.c_int64)]),
}


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load the library (building it first when absent and nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError(f"seismic_gb300: CUDA library missing at {LIB_PATH}; run build()")
        build()
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class SeisError(RuntimeError):
    """A non-zero status from the C ABI, with the engine's message."""

    def __init__(self, status: int, message: str):
        super().__init__(f"seis status {status}: {message}")
        self.status = status
