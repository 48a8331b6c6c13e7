"""Golden vectors of a whole L-BFGS inversion, run by the reference itself.

Run (where the reference checkout exists; about an hour on one core):

    python tests/golden/make_golden_inversion.py /path/to/jcottaar-seismic

Imports the reference's unmodified ``core/seis_invert.py`` (with
``seis_forward2``, ``seis_prior`` and ``seis_numerics``) through the NumPy shim
of ``tests/golden/_shim`` and runs ``InversionModel.seis_to_vel_lbfgs``
(core/seis_invert.py:109-152) in FP64 on the CPU: the reference's own cost
(core/seis_invert.py:19-49), its FP64 engine, its L-BFGS with strong-Wolfe line
search and its RowTotalVariation prior.  Tensors the reference allocates with
``device='cuda'`` (core/seis_invert.py:141, core/seis_numerics.py:336-340) are
CPU tensors of a subclass that reports ``is_cuda`` for the two-loop wrappers'
asserts (core/seis_numerics.py:584,616); nothing of the reference's arithmetic
changes.

Case: a seeded layered 70x70 model (the reference's geometry: 5 shots, nt=999,
70 receivers), its records as the observed data, and a start model smoothed
with a 4-cell Gaussian.  Writes ``tests/golden/ref70_lbfgs.npz``:

* ``true_vec``, ``start_vec`` (4901): the models (the observed data are the
  reference's records of ``true_vec``, which the FP64 oracle reproduces exactly);
* ``cg_*``: the reference's ``cost_and_gradient`` at the start point (cost,
  gradient over the 71 unknowns, prior and residual parts);
* ``final_vec``: the model ``seis_to_vel_lbfgs`` returns after ``maxiter``
  iterations; ``evals_cost`` / ``evals_residual``: cost and residual misfit of
  every evaluation in order (unscaled).
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

MODEL_SEED = 101
SMOOTH_CELLS = 4.0
MAXITER = 60


class _Seismogram:
    """The reference's record container as ``seis_to_vel_lbfgs`` uses it (``to_vector``)."""

    def __init__(self, vec):
        self.vec = vec

    def to_vector(self):
        return self.vec


class _Velocity:
    """The reference's model container as ``seis_to_vel_lbfgs`` uses it
    (``to_vector`` / ``from_vector`` / ``to_cupy``, core/kaggle_support.py:221-253)."""

    def __init__(self, vec):
        self.vec = vec

    def to_vector(self):
        return self.vec

    def from_vector(self, v):
        self.vec = v

    def to_cupy(self):
        pass


def main(ref_root):
    sys.path.insert(0, os.path.join(HERE, "_shim"))
    sys.path.insert(1, os.path.join(ref_root, "core"))
    sys.path.insert(0, ROOT)
    import torch

    class HostAsCuda(torch.Tensor):
        """CPU tensor that reports is_cuda; operations keep the subclass."""
        @property
        def is_cuda(self):
            return True

        def __deepcopy__(self, memo):
            return torch.Tensor(self).clone().as_subclass(HostAsCuda)

    real_zeros, real_tensor = torch.zeros, torch.tensor

    def on_cpu(fn):
        def f(*args, **kw):
            if kw.get("device") == "cuda":
                kw["device"] = "cpu"
            return fn(*args, **kw).as_subclass(HostAsCuda)
        return f

    import cupy as cp  # the shim
    import seis_forward2
    import seis_invert
    import seis_prior

    from seismic_gb300 import synthetic

    real_from_dlpack = seis_invert.from_dlpack
    seis_invert.from_dlpack = lambda x: real_from_dlpack(x).as_subclass(HostAsCuda)
    # the shim's arrays hand themselves to torch through DLPack (CuPy's toDlpack)
    cp.ndarray.toDlpack = lambda self: np.ascontiguousarray(np.asarray(self)).__dlpack__()

    rng = np.random.default_rng(MODEL_SEED)
    vt = synthetic.model(rng, "layered")
    v0 = synthetic.smoothed(vt, SMOOTH_CELLS)
    true_vec = synthetic.to_vector(vt)
    start_vec = synthetic.to_vector(v0, vt.min())
    t0 = time.time()
    target = np.asarray(seis_forward2.vel_to_seis(cp.array(true_vec[:, None]))[0])
    print(f"observed records: {time.time() - t0:.1f} s", flush=True)

    prior = seis_prior.RowTotalVariation()
    prior.prep()
    B = prior.basis_vectors
    x_start = np.linalg.solve(B.T @ B, B.T @ start_vec[:, None])
    t0 = time.time()
    c, g, cpr, cre = seis_invert.cost_and_gradient(cp.array(x_start), cp.array(target), prior, B,
                                                   compute_gradient=True)
    print(f"cost_and_gradient: {time.time() - t0:.1f} s", flush=True)
    out = dict(model_seed=MODEL_SEED, smooth_cells=SMOOTH_CELLS, maxiter=MAXITER, prior="RowTotalVariation",
               prior_lambda=float(prior.λ), prior_epsilon=float(prior.epsilon), scaling=1e15,
               true_vec=true_vec, start_vec=start_vec, x_start=x_start[:, 0],
               cg_cost=float(c), cg_grad=np.asarray(g)[:, 0], cg_cost_prior=float(cpr), cg_cost_residual=float(cre))

    evals = []
    real_cg = seis_invert.cost_and_gradient

    def recording_cg(*args, **kw):
        r = real_cg(*args, **kw)
        evals.append((float(r[0]), float(r[-1])))
        print(f"  evaluation {len(evals)}: cost {float(r[0]):.9e} residual {float(r[-1]):.9e} "
              f"({time.time() - t0:.0f} s)", flush=True)
        return r

    seis_invert.cost_and_gradient = recording_cg
    model = seis_invert.InversionModel(prior=prior)
    model._prior_in_use = prior
    torch.zeros, torch.tensor = on_cpu(real_zeros), on_cpu(real_tensor)
    t0 = time.time()
    try:
        res = model.seis_to_vel_lbfgs(_Seismogram(cp.array(target)), _Velocity(cp.array(start_vec[:, None])),
                                      maxiter=MAXITER)
    finally:
        torch.zeros, torch.tensor = real_zeros, real_tensor
        seis_invert.cost_and_gradient = real_cg
    print(f"seis_to_vel_lbfgs: {time.time() - t0:.1f} s, {len(evals)} evaluations", flush=True)
    out.update(final_vec=np.asarray(res.to_vector())[:, 0], evals_cost=np.array([e[0] for e in evals]),
               evals_residual=np.array([e[1] for e in evals]))
    np.savez_compressed(os.path.join(HERE, "ref70_lbfgs.npz"), **out)
    print("wrote ref70_lbfgs.npz")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SEISMIC_REFERENCE", ""))
