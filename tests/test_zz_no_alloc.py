"""The allocation-free forward entry point, ``seis_forward_noalloc``.

It exists for callers that cannot call cudaMalloc once they are running (a
host whose allocator already reserved the device's memory, a latency-critical
loop that may not take cudaMalloc's implicit synchronisation, a plugin host
that forbids allocation in its callbacks).  Its workspace is a fixed static
device array shared by all calls, so the GPU test calls it twice in a row on
different models -- the second call must not see the first call's state -- and
checks both records against the engine's regular entry point,
``seis_vel_to_seis``, at the records tolerance of the parity tests.  This file
is collected last so that a run stopping at the first failure has run every
other test first.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

REC_TOL = 1e-5


def _call(lib, geom, vec, out, stream):
    g, keep = geom.to_c()
    rc = lib.seis_forward_noalloc(ctypes.byref(g), ctypes.c_void_p(vec.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                  ctypes.c_void_p(stream))
    del keep
    return rc


@pytest.mark.gpu
def test_noalloc_matches_engine_on_two_calls_in_a_row():
    import torch

    from seismic_gb300 import _lib, synthetic
    from seismic_gb300.engine import Engine
    from seismic_gb300.geometry import Geometry

    assert torch.cuda.is_available()
    lib = _lib.load()
    g = Geometry.reference()
    vecs = [synthetic.to_vector(synthetic.model(np.random.default_rng(s), f))
            for s, f in [(101, "curved"), (102, "faulted")]]
    dev_vecs = [torch.as_tensor(v, device="cuda") for v in vecs]
    stream = torch.cuda.current_stream().cuda_stream
    outs = []
    for v in dev_vecs:                      # two calls in a row on the shared scratch
        out = torch.full((g.nrecords,), float("nan"), dtype=torch.float64, device="cuda")
        rc = _call(lib, g, v, out, stream)
        assert rc == 0, lib.seis_last_error(None)
        outs.append(out)
    torch.cuda.synchronize()
    eng = Engine(g, max_models=1)
    for v, out in zip(dev_vecs, outs):
        ref, _, _, _ = eng.vel_to_seis(v)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_l2(got, ref.cpu().numpy()[0]) < REC_TOL
    assert rel_l2(outs[0].cpu().numpy(), outs[1].cpu().numpy()) > 1e-3   # different models, different records
    eng.close()
    # host memory is refused, not handed to a kernel
    host_out = torch.empty(g.nrecords, dtype=torch.float64).pin_memory()
    assert _call(lib, g, dev_vecs[0], host_out, stream) == -1
    assert "device memory" in lib.seis_last_error(None).decode()


def test_noalloc_rejects_geometry_beyond_its_workspace():
    """A geometry needing more than SEIS_NOALLOC_SCRATCH_BYTES fails with a clear
    message before any device work (runs without a GPU)."""
    from seismic_gb300 import _lib
    from seismic_gb300.geometry import Geometry

    lib = _lib.load()
    g = Geometry.surface(350, 500, 10, 1000)
    c, keep = g.to_c()
    rc = lib.seis_forward_noalloc(ctypes.byref(c), ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    del keep
    assert rc == -1
    msg = lib.seis_last_error(None).decode()
    assert "bytes of scratch" in msg and str(8 << 20) in msg
