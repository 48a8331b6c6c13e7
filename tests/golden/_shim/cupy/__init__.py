"""NumPy stand-in for the subset of CuPy that the reference's FD engine uses.

Test infrastructure only: ``tests/golden/make_golden.py`` puts this directory
ahead of the reference's ``core/`` on ``sys.path`` so that the reference's own
``seis_forward2.py`` / ``seis_numerics.py`` run unmodified on the CPU in FP64
and produce golden vectors.

What is emulated:

* array creation / elementwise / reductions map straight to NumPy;
* ``cuda.Stream`` is a context manager whose ``begin_capture`` /
  ``end_capture`` RECORD the kernel calls issued while capturing and whose
  graph ``launch`` REPLAYS them in order (the reference captures each 999-step
  time loop once and replays it for every shot, with per-shot parameters held
  in buffers that the replay reads at launch time);
* ``RawModule(code).get_function(name)`` returns NumPy restatements of the
  reference's CUDA-C kernels (``core/seis_forward2.py:381-582`` and
  ``core/seis_numerics.py:450-565``) that follow each kernel's arithmetic in the
  same order.  Kernel arguments that the reference passes as "pointer + offset"
  arrive here as flat NumPy views, and each restatement touches only the first
  ``nx*ny`` (or ``n``) elements, as the kernels do.
"""
import numpy as _np

from . import cuda  # noqa: F401  (cp.cuda.Stream)
from ._kernels import KERNELS as _KERNELS

ndarray = _np.ndarray
float64 = _np.float64
float32 = _np.float32
int32 = _np.int32
int64 = _np.int64


def array(obj, dtype=None, copy=True):
    return _np.array(obj, dtype=dtype, copy=copy)


def asarray(obj, dtype=None):
    return _np.asarray(obj, dtype=dtype)


def asnumpy(obj):
    return _np.asarray(obj)


def copy(a):
    return _np.array(a, copy=True)


zeros = _np.zeros
zeros_like = _np.zeros_like
ones = _np.ones
empty = _np.empty
eye = _np.eye
arange = _np.arange
pad = _np.pad
reshape = _np.reshape
concatenate = _np.concatenate
sum = _np.sum  # noqa: A001
mean = _np.mean
sqrt = _np.sqrt
exp = _np.exp
abs = _np.abs  # noqa: A001
diff = _np.diff
min = _np.min  # noqa: A001
max = _np.max  # noqa: A001
all = _np.all  # noqa: A001
diag = _np.diag
linalg = _np.linalg


def from_dlpack(x):
    # torch CPU tensors (the L-BFGS path) share memory with the returned array
    return x.numpy() if hasattr(x, "numpy") else _np.from_dlpack(x)


class RawModule:
    """Returns NumPy restatements of the named kernels (see ``_kernels``)."""

    def __init__(self, code=None, options=(), name_expressions=()):
        self.code = code

    def get_function(self, name):
        fn = _KERNELS[name]
        return _Launcher(fn)


class _Launcher:
    def __init__(self, fn):
        self.fn = fn

    def __call__(self, grid, block, args, shared_mem=0):
        rec = cuda._capture_list()
        if rec is not None:
            rec.append((self.fn, args))
        else:
            self.fn(*args)
