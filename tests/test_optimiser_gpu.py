"""GPU: the device-resident L-BFGS with its strong-Wolfe line search (``seis_lbfgs_step``)
against the host-driven generators (``numerics.lbfgs`` / ``strong_wolfe``, restating
core/seis_numerics.py:138-448) run with the same reductions: the same points, bit for
bit, through bracketing, zoom and every stopping rule; and the batched L-BFGS inversion
with the optimiser on the device against the same inversion driven from the host."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as _t
    assert _t.cuda.is_available(), "GPU tests need CUDA"
    return _t


def _rosenbrock(torch, X, A):
    """Row-wise scaled Rosenbrock: f_p = sum_i (1 - x_i)^2 + a_p (x_{i+1} - x_i^2)^2 and its
    gradient, elementwise on the device; each row's sum is the library's fixed-order
    reduction, so a row's value does not depend on the batch."""
    from seismic_gb300 import numerics
    a = A[:, None]
    u = 1.0 - X[:, :-1]
    v = X[:, 1:] - X[:, :-1] ** 2
    terms = torch.zeros_like(X)
    terms[:, :-1] = u * u + a * (v * v)
    g = torch.zeros_like(X)
    g[:, :-1] = -2.0 * u - 4.0 * a * v * X[:, :-1]
    g[:, 1:] += 2.0 * a * v
    f = torch.stack([torch.tensor(numerics.DEVICE_OPS.sumabs(terms[p]), dtype=torch.float64, device=X.device)
                     for p in range(X.shape[0])])
    return f, g


@pytest.mark.parametrize("n,max_iter,tol_grad,tol_change", [(50, 30, 1e-7, 0.0), (300, 12, 1e-7, 0.0),
                                                            (50, 60, 1e-3, 1e-9), (20, 3, 1e-7, 0.0)])
def test_device_lbfgs_matches_host_generators(torch, n, max_iter, tol_grad, tol_change):
    from seismic_gb300 import numerics
    P = 5
    rng = np.random.default_rng(n + max_iter)
    X0 = torch.as_tensor(rng.normal(0.0, 1.2, (P, n)), device="cuda")
    A = torch.as_tensor([1.0, 10.0, 100.0, 3.0, 30.0], dtype=torch.float64, device="cuda")
    func = lambda X, rows: _rosenbrock(torch, X, A[rows])
    Xd, evals = numerics.bfgs_device(func, X0, max_iter, tol_grad, tol_change, poll_every=3)
    torch.cuda.synchronize()
    for p in range(P):
        def one(x, p=p):
            f, g = _rosenbrock(torch, x[None, :], A[p:p + 1])
            return float(f[0]), g[0]
        xh = numerics.bfgs(one, X0[p].clone(), max_iter, tol_grad, tol_change, ops=numerics.DEVICE_OPS)
        assert torch.equal(xh, Xd[p]), (p, float((xh - Xd[p]).abs().max()))
    f0, _ = func(X0, list(range(P)))
    f1, _ = func(Xd, list(range(P)))
    assert bool((f1 < f0).all())


def test_device_lbfgs_state_machine_edges(torch):
    """A problem already optimal at x0 stops after one evaluation; later steps leave
    finished problems untouched."""
    from seismic_gb300 import numerics
    X0 = torch.ones((2, 16), dtype=torch.float64, device="cuda")
    X0[1, 3] = 1.5
    A = torch.as_tensor([5.0, 5.0], dtype=torch.float64, device="cuda")
    opt = numerics.DeviceLBFGS(X0, 10, 1e-7, 0.0)
    f, g = _rosenbrock(torch, opt.x_eval, A)
    opt.step(f, g)
    assert opt.done.tolist() == [1, 0]
    for _ in range(80):
        f, g = _rosenbrock(torch, opt.x_eval, A)
        opt.step(f, g)
    assert opt.done.tolist() == [1, 1]
    assert torch.equal(opt.x_eval[0], X0[0])
    last = opt.x_eval.clone()
    opt.step(*_rosenbrock(torch, last, A))
    assert torch.equal(opt.x_eval, last)


def test_batched_lbfgs_inversion_device_loop(torch):
    """Three 70x70 models (5 shots, nt 300) with the TV prior: the device-resident
    optimiser gives the host-driven run's models bit for bit, and lowers the misfit."""
    from seismic_gb300 import inversion, priors, synthetic
    from seismic_gb300.engine import Engine
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=300)
    vecs, trues, _ = synthetic.batch(71, 3)
    eng = Engine(g, max_models=3)
    targets = eng.vel_to_seis(torch.as_tensor(trues, device="cuda"))[0]
    starts = torch.as_tensor(vecs, device="cuda")
    pr = priors.TotalVariation(70, 70, device="cuda").prep()
    out_d, ev = inversion.seis_to_vel_lbfgs_batched(targets, starts, pr, eng, maxiter=6, device_loop=True)
    out_h, _ = inversion.seis_to_vel_lbfgs_batched(targets, starts, pr, eng, maxiter=6, device_loop=False)
    assert torch.equal(out_d, out_h)
    mf0 = eng.vel_to_seis(starts, None, targets, adjoint_on_residual=True, want_misfit=True)[3]
    mf1 = eng.vel_to_seis(out_d, None, targets, adjoint_on_residual=True, want_misfit=True)[3]
    assert bool((mf1 < 0.5 * mf0).all()), (mf0, mf1)
    assert 6 <= ev <= 25 * 6 + 1


def test_batched_lbfgs_inversion_device_loop_rowtv_basis(torch):
    """The same with the RowTV prior (a basis of row profiles: N unknowns, not nv; the
    priors evaluated one request at a time) on a small grid, and the early stop on the
    records' misfit (seis_error_tolerance)."""
    from seismic_gb300 import inversion, priors, synthetic
    from seismic_gb300.engine import Engine
    from seismic_gb300.geometry import Geometry
    g = Geometry(nz=30, nx=40, nbc=30, nt=400, source_x_cells=(0, 13, 26, 39))
    rng = np.random.default_rng(73)
    trues = np.stack([synthetic.to_vector(synthetic.layered(rng, 30, 40)) for _ in range(3)])
    starts = np.stack([synthetic.to_vector(synthetic.smoothed(synthetic.layered(rng, 30, 40), 3.0)) for _ in range(3)])
    eng = Engine(g, max_models=3)
    targets = eng.vel_to_seis(torch.as_tensor(trues, device="cuda"))[0]
    st = torch.as_tensor(starts, device="cuda")
    pr = priors.RowTotalVariation(30, 40, device="cuda").prep()
    for tol in (0.0, 1e-9):
        out_d, _ = inversion.seis_to_vel_lbfgs_batched(targets, st, pr, eng, maxiter=8, device_loop=True,
                                                       seis_error_tolerance=tol)
        out_h, _ = inversion.seis_to_vel_lbfgs_batched(targets, st, pr, eng, maxiter=8, device_loop=False,
                                                       seis_error_tolerance=tol)
        assert torch.equal(out_d, out_h)
