"""Differentiable FD modelling for torch: ``vel_to_seis`` as a ``torch.autograd.Function``.

* forward  -- records F(v) of a batch of model vectors (the engine's forward sweep);
* backward -- J^T w with w the incoming gradient of the records: one engine call
  with ``vec_adjoint = w`` (the reference's ``vel_to_seis(vec, vec_adjoint=w)``,
  core/seis_forward2.py:146), which reruns the forward sweep with its history
  (or, with ``checkpoint_every=k``, keeps the wavefield every k steps and
  recomputes each segment) and then the adjoint sweep;
* jvp      -- J v for forward-mode AD (the tangent sweep, core/seis_forward2.py:469-513).

Inputs and outputs are FP64 (M, nz*nx+1) model vectors and (M, nshots*nt*nrec)
records on the engine's device, as everywhere in this package.
"""
from __future__ import annotations

import torch

from .engine import Engine
from .geometry import Geometry


class _VelToSeis(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vec: torch.Tensor, engine: Engine):
        res, _, _, _ = engine.vel_to_seis(vec.detach())
        ctx.engine = engine
        ctx.save_for_backward(vec)
        ctx.save_for_forward(vec)
        return res

    @staticmethod
    def backward(ctx, grad_records: torch.Tensor):
        (vec,) = ctx.saved_tensors
        _, _, grad, _ = ctx.engine.vel_to_seis(vec.detach(), None, grad_records.detach().contiguous(),
                                               adjoint_on_residual=False)
        return grad, None

    @staticmethod
    def jvp(ctx, vec_dot: torch.Tensor, _engine_dot=None):
        (vec,) = ctx.saved_tensors
        _, rd, _, _ = ctx.engine.vel_to_seis(vec.detach(), vec_dot.detach().contiguous())
        return rd


class SeismicModelling(torch.nn.Module):
    """Records of a batch of models, differentiable through the engine's sweeps.

    ``checkpoint_every``: keep the forward wavefield every k steps in the
    backward pass and recompute the segments (0 keeps the whole increment
    history, the fastest choice when it fits in memory)."""

    def __init__(self, geometry: Geometry, max_models: int = 1, checkpoint_every: int = 0,
                 max_shots_per_chunk: int = 0):
        super().__init__()
        self.geometry = geometry
        self.engine = Engine(geometry, max_models=max_models, max_shots_per_chunk=max_shots_per_chunk)
        if checkpoint_every:
            self.engine.set_option("checkpoint_every", checkpoint_every)

    def forward(self, vec: torch.Tensor) -> torch.Tensor:
        squeeze = vec.dim() == 1
        v = vec.reshape(1, -1) if squeeze else vec
        out = _VelToSeis.apply(v, self.engine)
        return out.reshape(-1) if squeeze else out


def vel_to_seis(vec: torch.Tensor, engine: Engine) -> torch.Tensor:
    """Differentiable records of (M, nv) model vectors with an existing engine."""
    return _VelToSeis.apply(vec, engine)
