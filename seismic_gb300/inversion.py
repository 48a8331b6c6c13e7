"""Full-waveform inversion on the GB300 engine: cost, gradient, Gauss-Newton and L-BFGS.

Restates jcottaar/seismic ``core/seis_invert.py`` over the engine (torch FP64
tensors on the engine's device; the sweeps run in the CUDA library):

| here | reference |
|---|---|
| ``cost_and_gradient`` | ``cost_and_gradient`` core/seis_invert.py:19-49 |
| ``seis_to_vel_gn`` (dense J, batched tangent columns) | ``InversionModel.seis_to_vel_gn`` :63-107 |
| ``seis_to_vel_gn_cg`` (matrix-free CG) | no counterpart: J^T J products by tangent + adjoint sweeps |
| ``seis_to_vel_gn_cg_batched`` | the same for many models at once, matvecs as fused ``gn_matvec`` calls |
| ``seis_to_vel_lbfgs`` | ``InversionModel.seis_to_vel_lbfgs`` :109-152 |
| ``seis_to_vel_lbfgs_batched`` | the same for many models at once, optimiser resident on the GPU |

Model vectors are (nv, 1) columns (nz*nx velocities + min_vel), records
(nrecords, 1), a basis B is (nv, N) with the unknowns x = (N, 1).
"""
from __future__ import annotations

import numpy as np
import torch

from . import numerics
from .engine import Engine

F64 = torch.float64


def _records(engine: Engine, vec: torch.Tensor) -> torch.Tensor:
    return engine.vel_to_seis(vec.reshape(1, -1))[0].reshape(-1, 1)


def cost_and_gradient(x, target, prior, basis_functions, engine: Engine, compute_gradient: bool = False):
    """prior(x) + mean((F(Bx) - t)^2) and, with compute_gradient, its gradient
    grad_prior + (2/len(t)) B^T J^T (F(Bx) - t).  Returns the reference's tuples:
    (cost, gradient, cost_prior, cost_residual) or (cost, cost_prior, cost_residual)."""
    if compute_gradient:
        cost_prior, gradient_prior = prior.compute_cost_and_gradient(x, compute_gradient=True)
    else:
        cost_prior = prior.compute_cost_and_gradient(x, compute_gradient=False)
    vec = basis_functions @ x
    n = target.numel()
    engine.poll()   # callers read each evaluation on the host: report an earlier call's failure
    if compute_gradient:
        s, _, s_adjoint, mf = engine.vel_to_seis(vec.reshape(1, -1), None, target.reshape(1, -1),
                                                 adjoint_on_residual=True, want_misfit=True)
        cost_residual = mf[0] / n
        gradient = gradient_prior + (2.0 / n) * (basis_functions.T @ s_adjoint.reshape(-1, 1))
        return cost_prior + cost_residual, gradient, cost_prior, cost_residual
    s = _records(engine, vec)
    cost_residual = torch.mean((s - target) ** 2)
    return cost_prior + cost_residual, cost_prior, cost_residual


def project(basis_functions, vec):
    """Least-squares coordinates of a model vector in the basis: solve(B^T B, B^T v)."""
    from .priors import IdentityBasis
    if isinstance(basis_functions, IdentityBasis):
        return vec.clone()
    return torch.linalg.solve(basis_functions.T @ basis_functions, basis_functions.T @ vec)


def _line_search_scales(engine, prior, basis, x, step, target, scales):
    """Misfit + prior at x + s*step for every scale, forward sweeps batched in one call."""
    vecs = torch.cat([(basis @ (x + float(s) * step)).reshape(1, -1) for s in scales])
    costs = []
    for i0 in range(0, len(scales), engine.max_models):
        recs, _, _, _ = engine.vel_to_seis(vecs[i0:i0 + engine.max_models])
        for j, s in enumerate(scales[i0:i0 + engine.max_models]):
            res = torch.mean((recs[j].reshape(-1, 1) - target) ** 2)
            costs.append(float(prior.compute_cost_and_gradient(x + float(s) * step) + res))
    return np.array(costs)


def seis_to_vel_gn(target, velocity_guess, prior, engine: Engine, scales=None):
    """One Gauss-Newton pass with the dense Jacobian in the prior's basis
    (core/seis_invert.py:63-107).  The reference builds J column by column
    with one tangent call each; here the columns are one batched tangent call
    (the engine's models are copies of the linearisation point).  Needs a
    prior with a precision matrix P."""
    B = prior.basis_vectors
    x_guess = project(B, velocity_guess)
    n = target.numel()
    _, _, adj, _ = engine.vel_to_seis((B @ x_guess).reshape(1, -1), None, target.reshape(1, -1),
                                      adjoint_on_residual=True)
    rhs = -(B.T @ adj.reshape(-1, 1)) / n
    rhs = rhs - torch.cat((prior.lam * prior.P @ x_guess[:-1, :], torch.zeros((1, 1), dtype=F64, device=B.device)))
    nb = B.shape[1]
    P = torch.zeros((nb, nb), dtype=F64, device=B.device)
    P[:-1, :-1] = prior.lam * prior.P
    cols = []
    vg = velocity_guess.reshape(1, -1)
    for i0 in range(0, nb, engine.max_models):
        i1 = min(nb, i0 + engine.max_models)
        _, diff, _, _ = engine.vel_to_seis(vg.expand(i1 - i0, -1).contiguous(), B[:, i0:i1].T.contiguous())
        cols.append(diff)
    J = torch.cat(cols).T                       # (nrecords, nb)
    A = P + (J.T @ J) / n
    del J
    res_inv = torch.linalg.solve(A, rhs)
    step_v = B @ res_inv
    scales = np.linspace(-0.1, 1.1, 50) if scales is None else scales
    costs = _line_search_scales(engine, prior, B, x_guess, res_inv, target, scales)
    engine.check()
    return velocity_guess + _best_scale(scales, costs) * step_v


def _best_scale(scales, costs) -> float:
    """Scale of the lowest cost.  Scales whose model is unstable give NaN costs and are
    skipped (the reference's np.argmin would return the first NaN); 0 if all are NaN."""
    if np.all(np.isnan(costs)):
        return 0.0
    return float(scales[int(np.nanargmin(costs))])


def seis_to_vel_gn_cg(target, velocity_guess, prior, engine: Engine, n_outer: int = 10, n_cg: int = 20,
                      scales=None, prior_hvp_eps: float = 1e-4):
    """Matrix-free Gauss-Newton: each outer iteration solves
    (J^T J / N + H_p / 2) dx = -(J^T r / N + g_p / 2) by conjugate gradients with
    ``n_cg`` matrix-vector products (a tangent sweep J v and an adjoint sweep
    J^T (J v) each; FP64 inner products), then takes the best of a batched
    line search along dx.  H_p v is the prior's gradient difference along v
    (exact for quadratic priors).  Returns (model vector, per-iteration costs)."""
    B = prior.basis_vectors
    n = target.numel()
    x = project(B, velocity_guess)
    history = []
    scales = np.linspace(0.0, 1.2, 25) if scales is None else scales
    for _ in range(n_outer):
        vec = (B @ x).reshape(1, -1)
        s, _, adj, mf = engine.vel_to_seis(vec, None, target.reshape(1, -1), adjoint_on_residual=True,
                                           want_misfit=True)
        c_p, g_p = prior.compute_cost_and_gradient(x, compute_gradient=True)
        history.append(float(c_p) + float(mf[0]) / n)
        b = -((B.T @ adj.reshape(-1, 1)) / n + 0.5 * g_p)

        def matvec(v):
            _, jv, _, _ = engine.vel_to_seis(vec, (B @ v).reshape(1, -1))
            _, _, jtjv, _ = engine.vel_to_seis(vec, None, jv, adjoint_on_residual=False)
            h = (B.T @ jtjv.reshape(-1, 1)) / n
            e = prior_hvp_eps
            gp = prior.compute_cost_and_gradient(x + e * v, compute_gradient=True)[1]
            gm = prior.compute_cost_and_gradient(x - e * v, compute_gradient=True)[1]
            return h + 0.25 * (gp - gm) / e

        dx = torch.zeros_like(x)
        r = b.clone()
        p = r.clone()
        rr = float((r * r).sum())
        for _k in range(n_cg):
            Ap = matvec(p)
            pAp = float((p * Ap).sum())
            if pAp <= 0:
                break
            a = rr / pAp
            dx = dx + a * p
            r = r - a * Ap
            rr_new = float((r * r).sum())
            if rr_new < 1e-30:
                break
            p = r + (rr_new / rr) * p
            rr = rr_new
        costs = _line_search_scales(engine, prior, B, x, dx, target, scales)
        x = x + _best_scale(scales, costs) * dx
    vec = (B @ x).reshape(-1, 1)
    _, _, _, mf = engine.vel_to_seis(vec.reshape(1, -1), None, target.reshape(1, -1), adjoint_on_residual=True,
                                     want_misfit=True)
    history.append(float(prior.compute_cost_and_gradient(x)) + float(mf[0]) / n)
    engine.check()
    return vec, history


def seis_to_vel_gn_cg_batched(targets, starts, prior, engine: Engine, n_outer: int = 10, n_cg: int = 20,
                              scales=None, prior_hvp_eps: float = 1e-4):
    """``seis_to_vel_gn_cg`` for M models of one geometry at once, sharing ``prior``
    (and its basis): every engine call carries all models -- the gradient, each
    CG matrix-vector product (one fused ``gn_matvec`` call: J v and J^T J v with a
    single forward sweep) and the line search (models x scales).  Each model runs
    its own CG (FP64 scalars; a model whose CG has converged or lost positive
    curvature keeps its step while the others continue), so the result for a
    model is the one ``seis_to_vel_gn_cg`` would give up to the stopping rule's
    batch dimension.  targets (M, nrecords), starts (M, nv); returns
    (models (M, nv), costs (n_outer + 1, M))."""
    B = prior.basis_vectors
    n = targets.shape[1]
    M = targets.shape[0]
    X = torch.stack([project(B, starts[i].reshape(-1, 1))[:, 0] for i in range(M)])     # (M, N)
    scales = np.linspace(0.0, 1.2, 25) if scales is None else scales
    history = []

    def model_vecs(Xm):
        return torch.stack([(B @ Xm[i].reshape(-1, 1))[:, 0] for i in range(Xm.shape[0])])

    def prior_grads(Xm):
        cs, gs = [], []
        for i in range(Xm.shape[0]):
            c, gr = prior.compute_cost_and_gradient(Xm[i].reshape(-1, 1), compute_gradient=True)
            cs.append(float(c))
            gs.append(gr[:, 0])
        return np.array(cs), torch.stack(gs)

    for _ in range(n_outer):
        V = model_vecs(X)
        _, _, adj, mf = engine.vel_to_seis(V, None, targets, adjoint_on_residual=True, want_misfit=True)
        cp, gp = prior_grads(X)
        history.append(cp + mf.cpu().numpy() / n)
        Bt_adj = torch.stack([(B.T @ adj[i].reshape(-1, 1))[:, 0] for i in range(M)])
        b = -(Bt_adj / n + 0.5 * gp)

        def matvec(Pm):
            _, _, jtjv = engine.gn_matvec(V, model_vecs(Pm))
            h = torch.stack([(B.T @ jtjv[i].reshape(-1, 1))[:, 0] for i in range(M)]) / n
            e = prior_hvp_eps
            return h + 0.25 * (prior_grads(X + e * Pm)[1] - prior_grads(X - e * Pm)[1]) / e

        dX = torch.zeros_like(X)
        R = b.clone()
        Pm = R.clone()
        rr = (R * R).sum(dim=1)
        live = torch.ones(M, dtype=torch.bool, device=X.device)
        for _k in range(n_cg):
            AP = matvec(Pm)
            pAp = (Pm * AP).sum(dim=1)
            live = live & (pAp > 0)
            if not bool(live.any()):
                break
            a = torch.where(live, rr / torch.where(live, pAp, torch.ones_like(pAp)), torch.zeros_like(pAp))
            dX = dX + a[:, None] * Pm
            R = R - a[:, None] * AP
            rr_new = (R * R).sum(dim=1)
            live = live & (rr_new >= 1e-30)
            beta = torch.where(live, rr_new / rr, torch.zeros_like(rr))
            Pm = torch.where(live[:, None], R + beta[:, None] * Pm, Pm)
            rr = torch.where(live, rr_new, rr)
            if not bool(live.any()):
                break
        # batched line search: all models x scales through the engine in max_models chunks
        trial = torch.cat([X + float(sc) * dX for sc in scales])          # (len(scales) * M, N)
        tv = model_vecs(trial)
        tg = targets.repeat(len(scales), 1)
        costs = np.empty(trial.shape[0])
        for i0 in range(0, trial.shape[0], engine.max_models):
            i1 = min(trial.shape[0], i0 + engine.max_models)
            recs, _, _, _ = engine.vel_to_seis(tv[i0:i1])
            res = torch.mean((recs - tg[i0:i1]) ** 2, dim=1).cpu().numpy()
            for j in range(i0, i1):
                costs[j] = float(prior.compute_cost_and_gradient(trial[j].reshape(-1, 1))) + res[j - i0]
        costs = costs.reshape(len(scales), M)
        best = torch.as_tensor([_best_scale(scales, costs[:, i]) for i in range(M)], dtype=X.dtype, device=X.device)
        X = X + best[:, None] * dX
    V = model_vecs(X)
    _, _, _, mf = engine.vel_to_seis(V, None, targets, adjoint_on_residual=True, want_misfit=True)
    history.append(prior_grads(X)[0] + mf.cpu().numpy() / n)
    engine.check()
    return V, np.array(history)


def seis_to_vel_lbfgs(target, velocity_guess, prior, engine: Engine, maxiter: int, scaling: float = 1e15,
                      tolerance_grad: float = 1e-7, tolerance_change: float = 0.0, seis_error_tolerance: float = 0.0):
    """L-BFGS from ``velocity_guess`` on prior(x) + mean((F(Bx)-t)^2) scaled by ``scaling``
    (core/seis_invert.py:109-152); a NaN result falls back to the starting model."""
    B = prior.basis_vectors
    x0 = project(B, velocity_guess)[:, 0].clone()

    def func(x):
        cost, grad, _cp, cr = cost_and_gradient(x[:, None], target, prior, B, engine, compute_gradient=True)
        if float(cr) < seis_error_tolerance:
            cost, grad = 0 * cost, 0 * grad
        return cost * scaling, grad[:, 0] * scaling

    x = numerics.bfgs(func, x0, maxiter, tolerance_grad, tolerance_change)
    engine.check()
    if torch.isnan(x).any():
        return velocity_guess.clone()
    return B @ x[:, None]


def seis_to_vel_lbfgs_batched(targets, velocity_guesses, prior, engine: Engine, maxiter: int,
                              scaling: float = 1e15, tolerance_grad: float = 1e-7, tolerance_change: float = 0.0,
                              seis_error_tolerance: float = 0.0, device_loop: bool = True, poll_every: int = 1):
    """``seis_to_vel_lbfgs`` for P models of one geometry at once: targets (P, nrecords),
    guesses (P, nv).  Every evaluation is one batched engine call plus the batched prior;
    with ``device_loop`` the optimiser runs on the GPU (``numerics.bfgs_device``: no host
    read per evaluation), else the host generators with the same reductions drive it
    (bitwise the same points).  Returns the final models (P, nv) and the evaluations."""
    from types import SimpleNamespace

    from .serving import batched_prior
    B = prior.basis_vectors
    P = targets.shape[0]
    n = engine.geometry.nrecords
    X0 = torch.stack([project(B, velocity_guesses[i].reshape(-1, 1))[:, 0] for i in range(P)])
    part = [SimpleNamespace(prior=prior)] * P
    tol = float(seis_error_tolerance)

    def func(X, rows):
        # every model's products with the basis on their own (a matrix-vector product each),
        # so that a model's evaluation does not depend on the batch it is in
        V = torch.stack([B @ X[i] for i in range(len(rows))])
        engine.poll()
        _, _, ra, mf = engine.vel_to_seis(V, None, targets[rows], adjoint_on_residual=True, want_misfit=True)
        cp, gp = batched_prior(part[:len(rows)], X)
        gp = torch.stack(gp) if isinstance(gp, list) else gp
        cost = (cp + mf / n) * scaling
        g = (gp + (2.0 / n) * torch.stack([B.T @ ra[i] for i in range(len(rows))])) * scaling
        if tol > 0:
            keep = (mf / n >= tol).to(cost.dtype)
            cost, g = cost * keep, g * keep[:, None]
        return cost, g

    if device_loop:
        X, evals = numerics.bfgs_device(func, X0, maxiter, tolerance_grad, tolerance_change, poll_every=poll_every)
    else:
        X, evals = torch.empty_like(X0), 0
        for i in range(P):
            def one(x, i=i):
                c, g = func(x[None, :], [i])
                return float(c[0]), g[0]
            X[i] = numerics.bfgs(one, X0[i], maxiter, tolerance_grad, tolerance_change, ops=numerics.DEVICE_OPS)
    engine.check()
    out = torch.stack([B @ X[i] for i in range(P)])
    bad = torch.isnan(X).any(dim=1)
    if bool(bad.any()):
        out[bad] = velocity_guesses[bad]
    return out, evals

