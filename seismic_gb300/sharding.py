"""Shot-sharded misfit and gradient across processes.

A model's shots are independent until the end of an evaluation, where the
reference adds every shot's contribution into one gradient
(core/seis_forward2.py:202-314).  With N ranks each rank sweeps a contiguous
share of the shots and one sum (misfit and the nz*nx+1 gradient) over the
process group completes the evaluation -- the only exchange of the path.
Replicas (independent models per rank, ``bench.py --gpus N``) need none.

``ShardedEvaluator`` runs the engine on the rank's shots; ``reduce_evaluation``
is the exchange, usable with any backend (NCCL on GPUs, gloo on CPU).
"""
from __future__ import annotations

from dataclasses import replace

import torch
import torch.distributed as dist

from .geometry import Geometry


def shard_shots(nshots: int, world: int, rank: int) -> range:
    """Contiguous block of shot indices of ``rank`` (sizes differ by at most one)."""
    base, extra = divmod(nshots, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def shot_subset(geometry: Geometry, shots) -> Geometry:
    """The geometry restricted to some of its shots (same grid, receivers, wavelet)."""
    cells = tuple(geometry.source_x_cells[i] for i in shots)
    return replace(geometry, source_x_cells=cells)


def record_slice(geometry: Geometry, shots: range) -> slice:
    """Where the records of a contiguous block of shots sit in the full record vector."""
    per = geometry.nt * geometry.nrec
    return slice(shots.start * per, shots.stop * per)


def reduce_evaluation(misfit: torch.Tensor, gradient: torch.Tensor, group=None):
    """Sum the ranks' misfits and gradients in place (one all-reduce of nv+1 values)."""
    buf = torch.cat((misfit.reshape(1), gradient.reshape(-1)))
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    misfit.copy_(buf[0].reshape(misfit.shape))
    gradient.copy_(buf[1:].reshape(gradient.shape))
    return misfit, gradient


class ShardedEvaluator:
    """Misfit sum((F(v)-t)^2) and its gradient J^T (F(v)-t) of one model, with this
    rank sweeping only its share of the shots; ``evaluate`` returns the totals.

    With more ranks than shots the ranks past the last shot hold no shots: they
    create no engine and add zeros to the sum, so every rank still joins the one
    all-reduce.  ``sweep`` replaces the engine for the rank's shots: a callable
    ``(local_geometry, vec (nv,), target (local records,)) -> (misfit, gradient (nv,))``
    (the engine's own sweep when None)."""

    def __init__(self, geometry: Geometry, rank: int | None = None, world: int | None = None, group=None,
                 sweep=None, **engine_kw):
        self.rank = dist.get_rank(group) if rank is None else rank
        self.world = dist.get_world_size(group) if world is None else world
        self.group = group
        self.geometry = geometry
        self.shots = shard_shots(geometry.nshots, self.world, self.rank)
        self.local = shot_subset(geometry, self.shots) if len(self.shots) else None
        self.engine = None
        if sweep is None and self.local is not None:
            from .engine import Engine
            self.engine = Engine(self.local, max_models=1, **engine_kw)
            sweep = self._engine_sweep
        self.sweep = sweep

    def _engine_sweep(self, local: Geometry, vec: torch.Tensor, target: torch.Tensor):
        self.engine.poll()
        _, _, grad, mf = self.engine.vel_to_seis(vec.reshape(1, -1), None, target.reshape(1, -1),
                                                 adjoint_on_residual=True, want_misfit=True)
        return mf[0], grad[0]

    def evaluate(self, vec: torch.Tensor, target: torch.Tensor):
        if self.local is None:
            mf = torch.zeros((), dtype=torch.float64, device=vec.device)
            grad = torch.zeros(self.geometry.nv, dtype=torch.float64, device=vec.device)
        else:
            t = target.reshape(-1)[record_slice(self.geometry, self.shots)]
            mf, grad = self.sweep(self.local, vec.reshape(-1), t)
            mf = torch.as_tensor(mf, dtype=torch.float64, device=vec.device).reshape(())
            grad = torch.as_tensor(grad, dtype=torch.float64, device=vec.device).reshape(-1)
        return reduce_evaluation(mf.clone(), grad.clone(), self.group)

    def close(self):
        if self.engine is not None:
            self.engine.close()
            self.engine = None
