"""Golden vectors of the reference's callers of the FD engine: priors and L-BFGS.

Run (where the reference checkout exists):

    python tests/golden/make_golden_callers.py /path/to/jcottaar-seismic

Imports the reference's unmodified ``core/seis_prior.py`` and
``core/seis_numerics.py`` through the NumPy shim of ``tests/golden/_shim``.
The reference's ``bfgs`` allocates its history with ``device='cuda'``
(core/seis_numerics.py:336-340); for this CPU run ``torch.zeros`` is wrapped to
map that device to the CPU.  Writes ``tests/golden/callers.npz``:

* priors: cost and gradient of RowTotalVariation, TotalVariation,
  SquaredExponential (identity basis and SVD transform) and RestrictFlatAreas
  at seeded points (lambda as set below);
* L-BFGS: the final iterate of ``bfgs`` on a seeded smooth test function
  (convex quadratic plus a quartic term) in 71 unknowns, 25 iterations.
"""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))


def test_function(n=71, seed=3):
    rng = np.random.default_rng(seed)
    A = rng.normal(0, 1, (n, n))
    Q = A @ A.T / n + np.eye(n)
    b = rng.normal(0, 1, n)
    x0 = rng.normal(0, 1, n)
    return Q, b, x0


def main(ref_root):
    sys.path.insert(0, os.path.join(HERE, "_shim"))
    sys.path.insert(1, os.path.join(ref_root, "core"))
    import seis_numerics
    import seis_prior

    out = {}
    rng = np.random.default_rng(0)
    # priors (lambda fixed so that costs are O(1))
    vel = 2000 + 500 * np.sin(np.arange(4900).reshape(70, 70) / 300.0)
    vel[:, 30:33] = 2600.0
    for name, mk in [("rowtv", lambda: seis_prior.RowTotalVariation()),
                     ("tv", lambda: seis_prior.TotalVariation()),
                     ("se", lambda: seis_prior.SquaredExponential())]:
        pr = mk()
        pr.λ = 1.0
        pr.prep()
        x = rng.normal(0, 1, (pr.N, 1)) * 50 + 2000
        c, g = pr.compute_cost_and_gradient(x, compute_gradient=True)
        out[f"{name}_x"], out[f"{name}_cost"], out[f"{name}_grad"] = x, np.asarray(c), np.asarray(g)
    pr = seis_prior.SquaredExponential()
    pr.transform = True
    pr.svd_cutoff = 1.0
    pr.λ = 1.0
    pr.prep()
    x = rng.normal(0, 1, (pr.N, 1))
    c, g = pr.compute_cost_and_gradient(x, compute_gradient=True)
    out["se_svd_N"], out["se_svd_x"], out["se_svd_cost"], out["se_svd_grad"] = pr.N, x, np.asarray(c), np.asarray(g)
    out["se_svd_basis_colnorms"] = np.linalg.norm(np.asarray(pr.basis_vectors), axis=0)

    class _Vel:
        data = vel
    pr = seis_prior.RestrictFlatAreas()
    pr.underlying_prior = seis_prior.TotalVariation()
    pr.underlying_prior.λ = 1.0
    pr.prep()
    pr.adapt(_Vel())
    x = rng.normal(0, 1, (pr.N, 1)) * 50 + 2000
    c, g = pr.compute_cost_and_gradient(x, compute_gradient=True)
    out["rfa_vel"], out["rfa_N"], out["rfa_x"], out["rfa_cost"], out["rfa_grad"] = vel, pr.N, x, np.asarray(c), np.asarray(g)

    # L-BFGS on a seeded smooth function
    Q, b, x0 = test_function()
    Qt, bt = torch.tensor(Q), torch.tensor(b)

    def f(x):
        r = Qt @ x
        return 0.5 * x @ r - bt @ x + 0.01 * (x ** 4).sum(), r - bt + 0.04 * x ** 3

    class HostAsCuda(torch.Tensor):
        """CPU tensor that reports is_cuda, for the wrappers' device asserts
        (core/seis_numerics.py:584,616); operations keep the subclass."""
        @property
        def is_cuda(self):
            return True

        def __deepcopy__(self, memo):
            return torch.Tensor(self).clone().as_subclass(HostAsCuda)

    real_zeros = torch.zeros

    def zeros_on_cpu(*args, **kw):
        if kw.get("device") == "cuda":
            kw["device"] = "cpu"
        return real_zeros(*args, **kw).as_subclass(HostAsCuda)
    torch.zeros = zeros_on_cpu
    try:
        xf = seis_numerics.bfgs(f, torch.tensor(x0.copy()).as_subclass(HostAsCuda), 25, 1e-12, 0.0)
    finally:
        torch.zeros = real_zeros
    out["lbfgs_x0"], out["lbfgs_xfinal"] = x0, torch.Tensor(xf).detach().numpy().copy()
    np.savez_compressed(os.path.join(HERE, "callers.npz"), **out)
    print("wrote callers.npz")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SEISMIC_REFERENCE", ""))
