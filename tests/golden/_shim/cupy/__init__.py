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

class ndarray(_np.ndarray):
    """NumPy array with CuPy's 0-d semantics: reductions and scalar indexing
    return 0-d arrays (``type(x.mean()) is cupy.ndarray``), which the
    reference's priors assert (core/seis_prior.py:54,60)."""

    def __array_wrap__(self, arr, context=None, return_scalar=False):
        return _np.asarray(arr).view(ndarray)

    def __getitem__(self, key):
        r = super().__getitem__(key)
        return r.view(ndarray) if isinstance(r, _np.ndarray) else _np.asarray(r).view(ndarray)


def _wrap(fn):
    def f(*args, **kw):
        r = fn(*args, **kw)
        return _np.asarray(r).view(ndarray)
    f.__name__ = getattr(fn, "__name__", "f")
    return f


float64 = _np.float64
float32 = _np.float32
int32 = _np.int32
int64 = _np.int64


def array(obj, dtype=None, copy=True):
    return _np.array(obj, dtype=dtype, copy=copy).view(ndarray)


def asarray(obj, dtype=None):
    return _np.asarray(obj, dtype=dtype).view(ndarray)


def asnumpy(obj):
    return _np.asarray(obj)


def copy(a):
    return _np.array(a, copy=True).view(ndarray)


zeros = _wrap(_np.zeros)
zeros_like = _wrap(_np.zeros_like)
ones = _wrap(_np.ones)
empty = _wrap(_np.empty)
eye = _wrap(_np.eye)
arange = _wrap(_np.arange)
pad = _wrap(_np.pad)
reshape = _wrap(_np.reshape)
concatenate = _wrap(_np.concatenate)
sum = _wrap(_np.sum)  # noqa: A001
mean = _wrap(_np.mean)
sqrt = _wrap(_np.sqrt)
exp = _wrap(_np.exp)
abs = _wrap(_np.abs)  # noqa: A001
diff = _wrap(_np.diff)
min = _wrap(_np.min)  # noqa: A001
max = _wrap(_np.max)  # noqa: A001
all = _wrap(_np.all)  # noqa: A001
diag = _wrap(_np.diag)


class linalg:  # noqa: N801
    inv = staticmethod(_wrap(_np.linalg.inv))
    solve = staticmethod(_wrap(_np.linalg.solve))

    @staticmethod
    def svd(a, full_matrices=True, compute_uv=True):
        r = _np.linalg.svd(_np.asarray(a), full_matrices=full_matrices, compute_uv=compute_uv)
        return tuple(_np.asarray(x).view(ndarray) for x in r) if compute_uv else _np.asarray(r).view(ndarray)


def from_dlpack(x):
    # torch CPU tensors and DLPack capsules of them (the L-BFGS path) share
    # memory with the returned array
    if hasattr(x, "numpy"):
        return x.numpy()
    if type(x).__name__ == "PyCapsule":
        import torch.utils.dlpack
        return torch.utils.dlpack.from_dlpack(x).numpy()
    return _np.from_dlpack(x)


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
