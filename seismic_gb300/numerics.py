"""L-BFGS with a strong-Wolfe line search, as resumable generators.

Restates the reference's optimiser (jcottaar/seismic ``core/seis_numerics.py``,
itself a port of torch 2.7's ``LBFGS``):

| here | reference |
|---|---|
| ``cubic_interpolate`` | ``_cubic_interpolate`` core/seis_numerics.py:279-304 |
| ``strong_wolfe`` (generator) | ``_strong_wolfe`` :138-277 |
| ``lbfgs`` (generator), ``bfgs`` (driver) | ``bfgs`` :307-448 |
| ``lbfgs_direction`` (CUDA two-loop) | ``lbfgs_backward`` / ``lbfgs_forward`` kernels :450-565 |
| ``DeviceLBFGS``, ``bfgs_device`` | the same optimiser resident on the GPU (``seis_lbfgs_step``) |

The generators yield the point to evaluate and receive ``(f, g)``: a caller can
drive one optimisation (``bfgs``) or interleave many and batch their
evaluations into one engine call (the serving loop).  Vectors are FP64 torch
tensors on the GPU; the two-loop recursion runs in the engine library
(``seis_lbfgs_direction``), with FP64 inner products.  The generators read each
inner product, |.| sum and maximum on the host, as the reference does
(core/seis_numerics.py:155,162,169,324); ``DeviceLBFGS`` runs the same control
flow on the device, many problems at once, with no host read per evaluation.
With ``ops=DEVICE_OPS`` the generators use the device optimiser's reductions and
give the same bits.
"""
from __future__ import annotations

import ctypes
import math

import torch

from ._lib import SeisError, load


class TorchOps:
    """Inner products and norms read back through torch (the reference's own reductions)."""

    @staticmethod
    def dot(a, b) -> float:
        return float(torch.dot(a, b))

    @staticmethod
    def sumabs(a) -> float:
        return float(a.abs().sum())

    @staticmethod
    def maxabs(a) -> float:
        return float(a.abs().max())


class DeviceOps:
    """The same through the library's fixed-order FP64 block reductions (``seis_reduce``),
    the ones the device-resident optimiser uses."""

    @staticmethod
    def _reduce(op: int, a, b=None) -> float:
        lib = load()
        out = torch.empty(1, dtype=torch.float64, device=a.device)
        st = torch.cuda.current_stream(a.device).cuda_stream
        vp = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
        rc = lib.seis_reduce(1, a.numel(), op, vp(a.contiguous()), vp(None if b is None else b.contiguous()), vp(out),
                             ctypes.c_void_p(st))
        if rc != 0:
            raise SeisError(rc, (lib.seis_last_error(None) or b"").decode())
        return float(out)

    @classmethod
    def dot(cls, a, b) -> float:
        return cls._reduce(0, a, b)

    @classmethod
    def sumabs(cls, a) -> float:
        return cls._reduce(1, a)

    @classmethod
    def maxabs(cls, a) -> float:
        return cls._reduce(2, a)


TORCH_OPS, DEVICE_OPS = TorchOps(), DeviceOps()


def cubic_interpolate(x1, f1, g1, x2, f2, g2, bounds=None):
    """Minimiser of the cubic through two points with function values and slopes."""
    if bounds is not None:
        xmin_bound, xmax_bound = bounds
    else:
        xmin_bound, xmax_bound = (x1, x2) if x1 <= x2 else (x2, x1)
    d1 = g1 + g2 - 3 * (f1 - f2) / (x1 - x2)
    d2_square = d1 * d1 - g1 * g2
    if d2_square >= 0:
        d2 = math.sqrt(d2_square)        # the reference's tensor sqrt: correctly rounded
        if x1 <= x2:
            min_pos = x2 - (x2 - x1) * ((g2 + d2 - d1) / (g2 - g1 + 2 * d2))
        else:
            min_pos = x1 - (x1 - x2) * ((g1 + d2 - d1) / (g1 - g2 + 2 * d2))
        return min(max(min_pos, xmin_bound), xmax_bound)
    return (xmin_bound + xmax_bound) / 2.0


def strong_wolfe(x, t, d, f, g, gtd, c1=1e-4, c2=0.9, tolerance_change=1e-9, max_ls=25, ops=TORCH_OPS):
    """Generator: yields x + t*d, receives (f_new, g_new); returns (f, g, t, evaluations)."""
    _dot = ops.dot
    d_norm = ops.maxabs(d)
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


def lbfgs(x0: torch.Tensor, max_iter: int, tolerance_grad: float, tolerance_change: float, lr: float = 1.0,
          ops=TORCH_OPS):
    """Generator form of the reference's ``bfgs``: yields points to evaluate, receives
    (f, g) with f a float and g a FP64 tensor; returns the final x."""
    _dot = ops.dot
    max_eval = max_iter * 5 // 4
    orig_loss, flat_grad = yield x0
    x = x0.clone()
    loss = float(orig_loss)
    current_evals = 1
    if ops.maxabs(flat_grad) <= tolerance_grad:
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
        t = min(1.0, 1.0 / ops.sumabs(flat_grad)) * lr if n_iter == 1 else lr
        gtd = _dot(flat_grad, d)
        x_init = x.clone()
        loss, flat_grad, t, ls_func_evals = yield from strong_wolfe(x_init, t, d, loss, flat_grad, gtd, ops=ops)
        x = x + t * d
        current_evals += ls_func_evals
        if n_iter == max_iter:
            break
        if current_evals >= max_eval:
            break
        if ops.maxabs(flat_grad) <= tolerance_grad:
            break
        if ops.maxabs(d * t) <= tolerance_change:
            break
        if abs(loss - prev_loss) < tolerance_change:
            break
    return x


def bfgs(cost_and_gradient_func, x0, max_iter, tolerance_grad, tolerance_change, ops=TORCH_OPS):
    """The reference's ``bfgs(cost_and_gradient_func, x0, max_iter, tol_grad, tol_change)``:
    ``cost_and_gradient_func(x) -> (cost, grad)``; returns the final x."""
    gen = lbfgs(x0, max_iter, tolerance_grad, tolerance_change, ops=ops)
    try:
        xq = next(gen)
        while True:
            f, g = cost_and_gradient_func(xq)
            xq = gen.send((float(f), g))
    except StopIteration as stop:
        return stop.value


class DeviceLBFGS:
    """L-BFGS with a strong-Wolfe line search for P problems of n unknowns, resident on
    the GPU (``seis_lbfgs_step``): the state machine of ``lbfgs`` / ``strong_wolfe`` with
    ``DEVICE_OPS``, advanced one evaluation at a time by one launch for all problems.

        opt = DeviceLBFGS(x0s, max_iter, tolerance_grad, tolerance_change)
        f, g = func(opt.x_eval)   # (P,), (P, n) FP64 on the device
        opt.step(f, g)            # no host read; opt.done (P,) int32 on the device

    A finished problem keeps its final x in ``x_eval`` and ignores later steps."""

    def __init__(self, x0s: torch.Tensor, max_iter: int, tolerance_grad: float, tolerance_change: float,
                 stream: torch.cuda.Stream | None = None):
        if x0s.device.type != "cuda" or x0s.dtype != torch.float64 or x0s.dim() != 2:
            raise ValueError("x0s must be a (P, n) FP64 CUDA tensor")
        self.lib = load()
        self.P, self.n = x0s.shape
        self.max_iter = int(max_iter)
        self.tol = (float(tolerance_grad), float(tolerance_change))
        nbytes = int(self.lib.seis_lbfgs_state_bytes(self.n, self.max_iter))
        if nbytes <= 0:
            raise ValueError("invalid sizes")
        self.state = torch.empty(self.P * nbytes + 256, dtype=torch.uint8, device=x0s.device)
        off = (-self.state.data_ptr()) % 256
        self._state_ptr = self.state.data_ptr() + off
        self.x_eval = torch.empty_like(x0s)
        self.done = torch.zeros(self.P, dtype=torch.int32, device=x0s.device)
        self.stream = stream
        self._call(x0s.contiguous(), None, None)

    def _call(self, x0, f, g):
        st = (self.stream or torch.cuda.current_stream(self.x_eval.device)).cuda_stream
        vp = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
        rc = self.lib.seis_lbfgs_step(self.P, self.n, self.max_iter, self.tol[0], self.tol[1], vp(x0), vp(f), vp(g),
                                      ctypes.c_void_p(self._state_ptr), vp(self.x_eval), vp(self.done),
                                      ctypes.c_void_p(st))
        if rc != 0:
            raise SeisError(rc, (self.lib.seis_last_error(None) or b"").decode())

    def step(self, f: torch.Tensor, g: torch.Tensor) -> None:
        """Consume f (P,) and g (P, n), the evaluation of the current ``x_eval``."""
        self._call(None, f.contiguous(), g.contiguous())


def bfgs_device(func, x0s: torch.Tensor, max_iter: int, tolerance_grad: float, tolerance_change: float,
                poll_every: int = 1, ahead: int = 2):
    """Device-resident ``bfgs`` of P problems at once: ``func(X, rows) -> (f (R,), g (R, n))``
    on the device, called once per evaluation round with the points X (R, n) of the
    problems ``rows`` (indices into the P problems).  The host never waits on an
    evaluation: completion is read through a pinned copy of the done flags, polled by CUDA
    event every ``poll_every`` rounds, and problems known to be done leave the rounds that
    follow (a problem's evaluation must not depend on the others in its round; those that
    finished but are not yet known to have are still evaluated, and ignore it).  The host
    queues at most ``ahead`` polled rounds beyond the device, which bounds those wasted
    evaluations while keeping the device busy.  Returns the final points and the number of
    rounds issued."""
    opt = DeviceLBFGS(x0s, max_iter, tolerance_grad, tolerance_change)
    P, dev = opt.P, x0s.device
    ring = [torch.zeros(P, dtype=torch.int32, pin_memory=True) for _ in range(ahead + 2)]
    fbuf = torch.zeros(P, dtype=torch.float64, device=dev)
    gbuf = torch.zeros_like(x0s)
    rows, idx = list(range(P)), None
    pending = []

    def seen(fl) -> bool:
        nonlocal rows, idx
        flags = fl.tolist()
        if all(flags):
            return True
        live = [i for i in range(P) if not flags[i]]
        if len(live) < len(rows):
            rows, idx = live, torch.tensor(live, dtype=torch.long, device=dev)
        return False

    # every iteration takes at most 25 line-search evaluations, plus the first one
    for k in range(25 * max_iter + 1):
        if idx is None:
            f, g = func(opt.x_eval, rows)
        else:
            fs, gs = func(opt.x_eval.index_select(0, idx), rows)
            fbuf.index_copy_(0, idx, fs)
            gbuf.index_copy_(0, idx, gs)
            f, g = fbuf, gbuf
        opt.step(f, g)
        if (k + 1) % poll_every == 0:
            ev = torch.cuda.Event()
            fl = ring[(k + 1) // poll_every % len(ring)]    # at most ahead + 1 polls in flight
            fl.copy_(opt.done, non_blocking=True)
            ev.record()
            pending.append((ev, fl))
        while pending and pending[0][0].query():
            _, fl = pending.pop(0)
            if seen(fl):
                return opt.x_eval.clone(), k + 1
        if len(pending) > ahead:      # keep the host at most `ahead` polls ahead of the device
            ev, fl = pending.pop(0)
            ev.synchronize()
            if seen(fl):
                return opt.x_eval.clone(), k + 1
    return opt.x_eval.clone(), 25 * max_iter + 1
