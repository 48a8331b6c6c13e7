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
    rank sweeping only its share of the shots; ``evaluate`` returns the totals."""

    def __init__(self, geometry: Geometry, rank: int | None = None, world: int | None = None, group=None,
                 **engine_kw):
        from .engine import Engine
        self.rank = dist.get_rank(group) if rank is None else rank
        self.world = dist.get_world_size(group) if world is None else world
        self.group = group
        self.geometry = geometry
        self.shots = shard_shots(geometry.nshots, self.world, self.rank)
        self.local = shot_subset(geometry, self.shots)
        self.engine = Engine(self.local, max_models=1, **engine_kw)

    def evaluate(self, vec: torch.Tensor, target: torch.Tensor):
        t = target.reshape(-1)[record_slice(self.geometry, self.shots)]
        _, _, grad, mf = self.engine.vel_to_seis(vec.reshape(1, -1), None, t.reshape(1, -1),
                                                 adjoint_on_residual=True, want_misfit=True)
        return reduce_evaluation(mf[0].clone(), grad[0].clone(), self.group)
