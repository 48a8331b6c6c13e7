"""L-BFGS with a strong-Wolfe line search, as resumable generators.

Restates the reference's optimiser (jcottaar/seismic ``core/seis_numerics.py``,
itself a port of torch 2.7's ``LBFGS``):

| here | reference |
|---|---|
| ``cubic_interpolate`` | ``_cubic_interpolate`` core/seis_numerics.py:279-304 |
| ``strong_wolfe`` (generator) | ``_strong_wolfe`` :138-277 |
| ``lbfgs`` (generator), ``bfgs`` (driver) | ``bfgs`` :307-448 |
| ``lbfgs_direction`` (CUDA two-loop) | ``lbfgs_backward`` / ``lbfgs_forward`` kernels :450-565 |

The generators yield the point to evaluate and receive ``(f, g)``: a caller can
drive one optimisation (``bfgs``) or interleave many and batch their
evaluations into one engine call (the serving loop).  Vectors are FP64 torch
tensors on the GPU; the two-loop recursion runs in the engine library
(``seis_lbfgs_direction``), with FP64 inner products.
"""
from __future__ import annotations

import ctypes

import torch

from ._lib import SeisError, load


def cubic_interpolate(x1, f1, g1, x2, f2, g2, bounds=None):
    """Minimiser of the cubic through two points with function values and slopes."""
    if bounds is not None:
        xmin_bound, xmax_bound = bounds
    else:
        xmin_bound, xmax_bound = (x1, x2) if x1 <= x2 else (x2, x1)
    d1 = g1 + g2 - 3 * (f1 - f2) / (x1 - x2)
    d2_square = d1 ** 2 - g1 * g2
    if d2_square >= 0:
        d2 = d2_square ** 0.5
        if x1 <= x2:
            min_pos = x2 - (x2 - x1) * ((g2 + d2 - d1) / (g2 - g1 + 2 * d2))
        else:
            min_pos = x1 - (x1 - x2) * ((g1 + d2 - d1) / (g1 - g2 + 2 * d2))
        return min(max(min_pos, xmin_bound), xmax_bound)
    return (xmin_bound + xmax_bound) / 2.0


def _dot(a, b) -> float:
    return float(torch.dot(a, b))


def strong_wolfe(x, t, d, f, g, gtd, c1=1e-4, c2=0.9, tolerance_change=1e-9, max_ls=25):
    """Generator: yields x + t*d, receives (f_new, g_new); returns (f, g, t, evaluations)."""
    d_norm = float(d.abs().max())
    g = g.clone()
    f_new, g_new = yield x + t * d
    ls_func_evals = 1
    gtd_new = _dot(g_new, d)
    t_prev, f_prev, g_prev, gtd_prev = 0.0, f, g, gtd
    done = False
    ls_iter = 0
    bracket = bracket_f = bracket_g = bracket_gtd = None
    while ls_iter < max_ls:
        if f_new > (f + c1 * t * gtd) or (ls_iter > 1 and f_new >= f_prev):
            bracket, bracket_f = [t_prev, t], [f_prev, f_new]
            bracket_g, bracket_gtd = [g_prev, g_new.clone()], [gtd_prev, gtd_new]
            break
        if abs(gtd_new) <= -c2 * gtd:
            bracket, bracket_f, bracket_g = [t], [f_new], [g_new]
            done = True
            break
        if gtd_new >= 0:
            bracket, bracket_f = [t_prev, t], [f_prev, f_new]
            bracket_g, bracket_gtd = [g_prev, g_new.clone()], [gtd_prev, gtd_new]
            break
        min_step = t + 0.01 * (t - t_prev)
        max_step = t * 10
        tmp = t
        t = cubic_interpolate(t_prev, f_prev, gtd_prev, t, f_new, gtd_new, bounds=(min_step, max_step))
        t_prev, f_prev, g_prev, gtd_prev = tmp, f_new, g_new.clone(), gtd_new
        f_new, g_new = yield x + t * d
        ls_func_evals += 1
        gtd_new = _dot(g_new, d)
        ls_iter += 1
    if ls_iter == max_ls:
        bracket, bracket_f, bracket_g = [0, t], [f, f_new], [g, g_new]
    insuf_progress = False
    low_pos, high_pos = (0, 1) if bracket_f[0] <= bracket_f[-1] else (1, 0)
    while not done and ls_iter < max_ls:
        if abs(bracket[1] - bracket[0]) * d_norm < tolerance_change:
            break
        t = cubic_interpolate(bracket[0], bracket_f[0], bracket_gtd[0], bracket[1], bracket_f[1], bracket_gtd[1])
        eps = 0.1 * (max(bracket) - min(bracket))
        if min(max(bracket) - t, t - min(bracket)) < eps:
            if insuf_progress or t >= max(bracket) or t <= min(bracket):
                if abs(t - max(bracket)) < abs(t - min(bracket)):
                    t = max(bracket) - eps
                else:
                    t = min(bracket) + eps
                insuf_progress = False
            else:
                insuf_progress = True
        else:
            insuf_progress = False
        f_new, g_new = yield x + t * d
        ls_func_evals += 1
        gtd_new = _dot(g_new, d)
        ls_iter += 1
        if f_new > (f + c1 * t * gtd) or f_new >= bracket_f[low_pos]:
            bracket[high_pos], bracket_f[high_pos] = t, f_new
            bracket_g[high_pos], bracket_gtd[high_pos] = g_new.clone(), gtd_new
            low_pos, high_pos = (0, 1) if bracket_f[0] <= bracket_f[1] else (1, 0)
        else:
            if abs(gtd_new) <= -c2 * gtd:
                done = True
            elif gtd_new * (bracket[high_pos] - bracket[low_pos]) >= 0:
                bracket[high_pos], bracket_f[high_pos] = bracket[low_pos], bracket_f[low_pos]
                bracket_g[high_pos], bracket_gtd[high_pos] = bracket_g[low_pos], bracket_gtd[low_pos]
            bracket[low_pos], bracket_f[low_pos] = t, f_new
            bracket_g[low_pos], bracket_gtd[low_pos] = g_new.clone(), gtd_new
    return bracket_f[low_pos], bracket_g[low_pos], bracket[low_pos], ls_func_evals


def lbfgs_direction(old_stps, old_dirs, ro, al, num_old: int, grad, h_diag: float) -> torch.Tensor:
    """d = -H g by the two-loop recursion over the first ``num_old`` stored pairs
    (one CUDA block, FP64 reductions).  Writes al[:num_old]."""
    n = grad.numel()
    d = torch.empty_like(grad)
    if grad.device.type != "cuda":
        raise RuntimeError("lbfgs_direction needs CUDA tensors (no CPU fallback)")
    lib = load()
    nold = torch.tensor([num_old], dtype=torch.int32, device=grad.device)
    hd = torch.tensor([h_diag], dtype=torch.float64, device=grad.device)
    st = torch.cuda.current_stream(grad.device).cuda_stream
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    rc = lib.seis_lbfgs_direction(1, n, old_stps.shape[0], vp(nold), vp(old_stps), vp(old_dirs), vp(ro), vp(al),
                                  vp(grad), vp(hd), vp(d), ctypes.c_void_p(st))
    if rc != 0:
        raise SeisError(rc, (lib.seis_last_error(None) or b"").decode())
    return d


def lbfgs(x0: torch.Tensor, max_iter: int, tolerance_grad: float, tolerance_change: float, lr: float = 1.0):
    """Generator form of the reference's ``bfgs``: yields points to evaluate, receives
    (f, g) with f a float and g a FP64 tensor; returns the final x."""
    max_eval = max_iter * 5 // 4
    orig_loss, flat_grad = yield x0
    x = x0.clone()
    loss = float(orig_loss)
    current_evals = 1
    if float(flat_grad.abs().max()) <= tolerance_grad:
        return x
    n_iter = 0
    prev_flat_grad = None
    cur_index = 0
    dev = x.device
    ro = torch.zeros(max_iter + 1, dtype=torch.float64, device=dev)
    al = torch.zeros(max_iter + 1, dtype=torch.float64, device=dev)
    old_dirs = torch.zeros(max_iter + 1, x.shape[0], dtype=torch.float64, device=dev)
    old_stps = torch.zeros(max_iter + 1, x.shape[0], dtype=torch.float64, device=dev)
    d = None
    t = None
    h_diag = 1.0
    while n_iter < max_iter:
        n_iter += 1
        if n_iter == 1:
            d = -flat_grad
            h_diag = 1.0
        else:
            y = flat_grad - prev_flat_grad
            s = d * t
            ys = _dot(y, s)
            if ys > 1e-10:
                old_dirs[cur_index, :] = y
                old_stps[cur_index, :] = s
                ro[cur_index] = 1.0 / ys
                cur_index += 1
                h_diag = ys / _dot(y, y)
            d = lbfgs_direction(old_stps, old_dirs, ro, al, cur_index, flat_grad, h_diag)
        prev_flat_grad = flat_grad.clone()
        prev_loss = loss
        t = min(1.0, 1.0 / float(flat_grad.abs().sum())) * lr if n_iter == 1 else lr
        gtd = _dot(flat_grad, d)
        x_init = x.clone()
        loss, flat_grad, t, ls_func_evals = yield from strong_wolfe(x_init, t, d, loss, flat_grad, gtd)
        x = x + t * d
        current_evals += ls_func_evals
        if n_iter == max_iter:
            break
        if current_evals >= max_eval:
            break
        if float(flat_grad.abs().max()) <= tolerance_grad:
            break
        if float((d * t).abs().max()) <= tolerance_change:
            break
        if abs(loss - prev_loss) < tolerance_change:
            break
    return x


def bfgs(cost_and_gradient_func, x0, max_iter, tolerance_grad, tolerance_change):
    """The reference's ``bfgs(cost_and_gradient_func, x0, max_iter, tol_grad, tol_change)``:
    ``cost_and_gradient_func(x) -> (cost, grad)``; returns the final x."""
    gen = lbfgs(x0, max_iter, tolerance_grad, tolerance_change)
    try:
        xq = next(gen)
        while True:
            f, g = cost_and_gradient_func(xq)
            xq = gen.send((float(f), g))
    except StopIteration as stop:
        return stop.value
