"""Generate the golden vectors of the FD engine from the reference itself.

Run (in a container where the reference checkout exists):

    python tests/golden/make_golden.py /path/to/jcottaar-seismic [output dir]

The reference's own ``core/seis_forward2.py`` and ``core/seis_numerics.py`` are
imported UNMODIFIED; only CuPy (absent here) is replaced by the NumPy shim in
``tests/golden/_shim`` (graph capture recorded and replayed, RawModule kernels
restated in NumPy), and ``kaggle_support`` by a stub of its dtype globals.
The run is FP64, the reference's own precision (core/kaggle_support.py:80-82).

Each case stores the inputs needed to regenerate the call (model vector,
tangent direction, seeds of the adjoint input) and the outputs:
every 10th record row of ``result`` / ``result_diff`` (the whole records do
not fit a small fixture), the sum and the sum of squares of EVERY record row
(shot, time step) and of the whole vectors, and the whole gradient
``result_adjoint``.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

ROW_STRIDE = 10
CASES = [
    # name, family, model seed, tangent seed (None: no tangent), adjoint seed, sigma_w, on_residual
    ("ref70_layered", "layered", 11, 12, 13, 1e-2, False),
    ("ref70_faulted_residual", "faulted", 21, None, 22, 1e-2, True),
]


def adjoint_input(seed: int, sigma: float, n: int) -> np.ndarray:
    return np.random.default_rng(seed).normal(0.0, sigma, (n, 1))


def tangent_input(seed: int, n: int) -> np.ndarray:
    return np.random.default_rng(seed).normal(0.0, 1.0, (n, 1))


def main(ref_root: str, out_dir: str = HERE):
    sys.path.insert(0, os.path.join(HERE, "_shim"))
    sys.path.insert(1, os.path.join(ref_root, "core"))
    sys.path.insert(0, ROOT)
    import seis_forward2  # the reference module, via the shim

    from seismic_gb300 import synthetic

    for name, fam, mseed, dseed, aseed, sigma, resid in CASES:
        v = synthetic.model(np.random.default_rng(mseed), fam)
        vec = synthetic.to_vector(v)[:, None]
        vd = tangent_input(dseed, vec.shape[0]) if dseed is not None else None
        w = adjoint_input(aseed, sigma, 5 * 999 * 70)
        t0 = time.time()
        res, rd, ra = seis_forward2.vel_to_seis(vec, vd, w, adjoint_on_residual=resid)
        print(f"{name}: reference run {time.time() - t0:.1f} s")
        rec = res.reshape(5, 999, 70)
        out = dict(vec=vec[:, 0], model_seed=mseed, family=fam, adjoint_seed=aseed, adjoint_sigma=sigma,
                   adjoint_on_residual=resid, row_stride=ROW_STRIDE,
                   rec_rows=rec[:, ::ROW_STRIDE, :], rec_sum=res.sum(), rec_sumsq=(res ** 2).sum(),
                   rec_row_sum=rec.sum(axis=2), rec_row_sumsq=(rec ** 2).sum(axis=2),
                   grad=ra[:, 0])
        if vd is not None:
            drec = rd.reshape(5, 999, 70)
            out.update(tangent_seed=dseed, drec_rows=drec[:, ::ROW_STRIDE, :], drec_sum=rd.sum(),
                       drec_sumsq=(rd ** 2).sum(), drec_row_sum=drec.sum(axis=2),
                       drec_row_sumsq=(drec ** 2).sum(axis=2))
        np.savez_compressed(os.path.join(out_dir, f"{name}.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SEISMIC_REFERENCE", ""),
         sys.argv[2] if len(sys.argv) > 2 else HERE)
