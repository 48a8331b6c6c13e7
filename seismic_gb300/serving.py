"""Continuous-batching service for whole inversions (L-BFGS + prior) on one GPU.

A request is one full inversion: target records, a starting model, a prior
(whose basis defines the unknowns) and an L-BFGS budget, run as
``seis_invert.seis_to_vel_lbfgs`` does (jcottaar/seismic core/seis_invert.py:109-152).
Each request's optimiser is a resumable generator (``numerics.lbfgs``); the
server advances all of them in lock-step *ticks*:

1. admit waiting requests whose arrival time has passed, in order, while their
   HBM footprint (engine workspace share + optimiser state + records) fits the
   budget -- requests arriving while others run join at the next tick;
2. group the active requests by geometry; each group's pending evaluation
   points go into ONE batched engine call (cost + gradient of every model of
   the group), issued on the group's own CUDA stream so that groups of
   different grid sizes overlap on the device;
3. hand each request its (cost, gradient) and advance its generator; finished
   requests free their memory at once.

Results do not depend on the batch mix: the engine computes each model's
records and gradient identically whatever else is in the call (tested).

``run_plain`` is the one-at-a-time form with the same code, for comparison.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import numerics
from .engine import Engine, vel_to_seis_multi
from .geometry import Geometry
from .inversion import project


@dataclass
class InversionRequest:
    rid: int
    geometry: Geometry
    target: torch.Tensor            # (nrecords,) FP64
    start: torch.Tensor             # (nv,) FP64 starting model vector
    prior: object                   # prepped prior; its basis defines the unknowns
    maxiter: int = 50
    scaling: float = 1e15
    tolerance_grad: float = 1e-7
    tolerance_change: float = 0.0
    seis_error_tolerance: float = 0.0   # stop once mean((F(v)-t)^2) is below (core/seis_invert.py:130-133)
    arrival: float = 0.0            # seconds after the start of the run
    # filled by the server
    result: torch.Tensor | None = None
    admitted: float = math.nan
    finished: float = math.nan
    evaluations: int = 0
    footprint: int = 0
    _gen: object = field(default=None, repr=False)
    _pending: torch.Tensor | None = field(default=None, repr=False)
    _x0: torch.Tensor | None = field(default=None, repr=False)
    _lane: int = field(default=0, repr=False)

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def geometry_key(g: Geometry) -> tuple:
    return (g.nz, g.nx, g.nbc, g.nt, g.dx, g.dt, g.freq, tuple(g.src_z), tuple(g.src_x), tuple(g.rec_z),
            tuple(g.rec_x))


def shot_workspace_bytes(g: Geometry, checkpoint_every: int = 0) -> int:
    """Device bytes the engine holds per concurrently swept shot for a gradient."""
    NZ, NX = g.padded_shape
    NP = NZ * ((NX + 31) // 32 * 32)
    if checkpoint_every:
        levels = 2 * math.ceil(g.nt / checkpoint_every) + checkpoint_every + 1
    else:
        levels = g.nt + 1
    return 4 * NP * (levels + 15)


def request_footprint(req: InversionRequest, checkpoint_every: int = 0, max_shots: int | None = None) -> int:
    """Device bytes a request holds: its optimiser state, records and vectors, and the
    sweep workspace of its shots (of at most ``max_shots``: the engine sweeps no more at
    once)."""
    g = req.geometry
    n = req.prior.N
    opt = 8 * (2 * (req.maxiter + 1) * n + 2 * (req.maxiter + 1) + 8 * n)
    shots = g.nshots if max_shots is None else min(g.nshots, max_shots)
    return shots * shot_workspace_bytes(g, checkpoint_every) + opt + 8 * 3 * g.nrecords + 8 * g.nv * 4


class _Group:
    """Engine + streams of one geometry lane.  The engine sweeps at most
    ``workspace_bytes`` worth of shots at a time (larger batches run in chunks within
    one call).  ``share``: a lane of the same geometry whose engine this lane uses too;
    the engine's calls then queue on that lane's engine stream (one call at a time,
    each with the GPU to itself), while each lane's optimiser work runs on its own
    stream."""

    def __init__(self, geometry: Geometry, max_models: int, checkpoint_every: int, device,
                 workspace_bytes: int | None = None, shared_gpu: bool = False, share: "_Group | None" = None):
        self.geometry = geometry
        self.stream = torch.cuda.Stream(device=device)
        self.checkpoint_every = checkpoint_every
        if share is not None:
            self.engine, self.engine_stream, self.owner = share.engine, share.engine_stream, False
            return
        self.owner = True
        self.engine_stream = torch.cuda.Stream(device=device)
        slots = max_models * geometry.nshots
        if workspace_bytes is not None:
            per_shot = shot_workspace_bytes(geometry, checkpoint_every)
            slots = max(1, min(slots, int(workspace_bytes // per_shot)))
        self.engine = Engine(geometry, max_models=max_models, max_shots_per_chunk=slots, device=device)
        if checkpoint_every:
            self.engine.set_option("checkpoint_every", checkpoint_every)
        if shared_gpu:
            # other engines' sweeps run at the same time: the SMs a cluster sweep leaves
            # free are not idle, so no side sweeps beside it
            self.engine.set_option("fwd_side", 0)
            self.engine.set_option("adj_side", 0)

    def call(self, vecs, targets):
        """One batched cost + gradient call: queued on the engine stream after the lane's
        own work, its outputs handed back to the lane's stream."""
        es = self.engine_stream
        es.wait_stream(self.stream)
        with torch.cuda.stream(es):
            _, _, grad, mf = self.engine.vel_to_seis(vecs, None, targets, adjoint_on_residual=True,
                                                     want_misfit=True, stream=es)
        for t in (vecs, targets):
            t.record_stream(es)
        self.stream.wait_stream(es)
        for t in (grad, mf):
            t.record_stream(self.stream)
        return grad, mf


class InversionServer:
    """Admission by HBM footprint, per-geometry batched evaluations, continuous batching.

    The admitted requests' footprints never exceed ``hbm_budget_bytes``; each of
    up to ``max_geometries`` geometries has ``lanes`` lanes, each with its own
    stream.  A geometry's requests are spread over its lanes, so one lane's
    host-side optimiser steps overlap the other lanes' sweeps.  The lanes of a
    geometry share one engine (``share_lane_engines``, the default when one geometry
    is served): its calls queue one after another, each with the whole GPU and its
    side sweeps; otherwise each lane has its own engine and their calls overlap on
    the device.  Engines split the budget equally for their sweep workspace, kept
    across calls.

    A geometry keeps whole forward histories when a chunk of shots that fills the GPU
    (``fill_shots``) fits its engine's share, else it uses checkpointed adjoints (every
    ``checkpoint_every`` steps); ``checkpoint_above_bytes`` instead checkpoints every
    geometry whose whole-history workspace per shot exceeds it."""

    def __init__(self, hbm_budget_bytes: int, max_batch: int = 64, device=None,
                 checkpoint_above_bytes: int | None = None, checkpoint_every: int = 50, max_geometries: int = 4,
                 lanes: int = 2, share_lane_engines: bool | None = None):
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.budget = int(hbm_budget_bytes)
        self.max_geometries = max_geometries
        self.lanes = lanes
        # one engine per geometry shared by its lanes when a single geometry is served (its
        # calls then have the GPU to themselves and run side sweeps); one per lane when
        # several geometries' calls overlap on the device
        self.share_lanes = max_geometries == 1 if share_lane_engines is None else share_lane_engines
        self.max_batch = max_batch
        self.checkpoint_above = checkpoint_above_bytes
        self.checkpoint_every = checkpoint_every
        self._ck: dict[tuple, int] = {}
        self.groups: dict[tuple, _Group] = {}
        self.active: list[InversionRequest] = []
        self.used = 0
        self.ticks = 0
        self.engine_calls = 0
        self.max_active = 0
        self.tick_s: list[float] = []

    # ------------------------------------------------------------------
    def _engine_share(self) -> int:
        """Sweep workspace of each engine: an equal share of the budget."""
        return self.budget // (self.max_geometries * (1 if self.share_lanes else self.lanes))

    def _ck_for(self, g: Geometry) -> int:
        if self.checkpoint_above is not None:
            return self.checkpoint_every if shot_workspace_bytes(g, 0) > self.checkpoint_above else 0
        key = geometry_key(g)
        if key not in self._ck:
            whole = fill_shots(g, self.device)[0] * shot_workspace_bytes(g, 0) <= self._engine_share()
            self._ck[key] = 0 if whole else self.checkpoint_every
        return self._ck[key]

    def _group(self, g: Geometry, lane: int) -> _Group:
        key = (geometry_key(g), lane)
        grp = self.groups.get(key)
        if grp is None:
            # each lane's engine sweeps within an equal share of the budget; a call
            # whose requests exceed it runs in several chunks
            share = self._group(g, 0) if self.share_lanes and lane > 0 else None
            engines = self.max_geometries * (1 if self.share_lanes else self.lanes)
            grp = _Group(g, self.max_batch, self._ck_for(g), self.device, workspace_bytes=self._engine_share(),
                         shared_gpu=engines > 1, share=share)
            self.groups[key] = grp
        return grp

    def _pick_lane(self, g: Geometry) -> int | None:
        """The least-loaded lane of the geometry with room for one more request."""
        gk = geometry_key(g)
        load = [0] * self.lanes
        for r in self.active:
            if geometry_key(r.geometry) == gk:
                load[r._lane] += 1
        lane = min(range(self.lanes), key=lambda i: load[i])
        return lane if load[lane] < self.max_batch else None

    def footprint(self, req: InversionRequest) -> int:
        g = req.geometry
        ck = self._ck_for(g)
        return request_footprint(req, ck, max(1, self._engine_share() // shot_workspace_bytes(g, ck)))

    def close(self):
        """Release the engines' device memory."""
        for grp in self.groups.values():
            if grp.owner:
                grp.engine.close()
        self.groups.clear()

    def _admit(self, req: InversionRequest, now: float, lane: int):
        req._lane = lane
        grp = self._group(req.geometry, lane)
        req.footprint = self.footprint(req)
        self.used += req.footprint
        req.admitted = now
        # the request's tensors were made on the caller's stream
        grp.stream.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(grp.stream):
            B = req.prior.basis_vectors
            req._x0 = project(B, req.start.reshape(-1, 1))[:, 0].clone()
            req._gen = numerics.lbfgs(req._x0, req.maxiter, req.tolerance_grad, req.tolerance_change)
            req._pending = next(req._gen)
        self.active.append(req)

    def _finish(self, req: InversionRequest, x: torch.Tensor, now: float):
        B = req.prior.basis_vectors
        req.result = req.start.clone() if torch.isnan(x).any() else (B @ x[:, None])[:, 0]
        req.finished = now
        req._gen = None
        req._pending = None
        self.used -= req.footprint

    # ------------------------------------------------------------------
    def _launch(self, grp: _Group, part: list):
        """Issue one batched cost + gradient call for ``part`` on the group's stream."""
        with torch.cuda.stream(grp.stream):
            vecs = torch.stack([(r.prior.basis_vectors @ r._pending[:, None])[:, 0] for r in part])
            tg = torch.stack([r.target for r in part])
            grad, mf = grp.call(vecs, tg)
            ev = torch.cuda.Event()
            ev.record(grp.stream)
        self.engine_calls += 1
        return (part, grad, mf, ev)

    def _complete(self, grp: _Group, flight, clock):
        """Hand each request of a finished call its (cost, gradient); advance its optimiser."""
        part, grad, mf, _ = flight
        grp.engine.poll()      # the call has completed: a timed-out bounded wait raises here
        done = []
        with torch.cuda.stream(grp.stream):
            n = grp.geometry.nrecords
            costs_p, grads_p = batched_prior(part, [r._pending for r in part])
            for i, r in enumerate(part):
                cost = (costs_p[i] + mf[i] / n) * r.scaling
                g = (grads_p[i] + (2.0 / n) * (r.prior.basis_vectors.T @ grad[i])) * r.scaling
                if r.seis_error_tolerance > 0 and float(mf[i]) / n < r.seis_error_tolerance:
                    cost, g = 0 * cost, 0 * g       # converged on the records: the optimiser stops
                r.evaluations += 1
                try:
                    r._pending = r._gen.send((float(cost), g))
                except StopIteration as stop:
                    done.append((r, stop.value))
        now = clock()
        for r, x in done:
            self._finish(r, x, now)
            self.active.remove(r)

    def run(self, requests: list[InversionRequest], realtime: bool = True) -> dict:
        """Serve ``requests`` (their ``arrival`` offsets in seconds).  With realtime, a
        request is admitted only once its arrival time has passed on the wall clock;
        otherwise every request is taken to arrive at time 0 (its ``arrival`` is reset).

        Each geometry group runs its own cycle: as soon as its previous batched call
        has completed (CUDA event), the group advances its requests and launches the
        next call with every active request of that geometry, so small grids are not
        held back by large ones and the groups' calls overlap on the device."""
        if not realtime:
            for r in requests:
                r.arrival = 0.0
        self.ticks = self.engine_calls = self.max_active = 0
        waiting = sorted(requests, key=lambda r: r.arrival)
        flights: dict[tuple, object] = {}
        t0 = time.perf_counter()

        def clock():
            return time.perf_counter() - t0

        while waiting or self.active or flights:
            now = clock()
            while waiting and (not realtime or waiting[0].arrival <= now):
                fp = self.footprint(waiting[0])
                if fp > self.budget:
                    raise ValueError(f"request {waiting[0].rid} needs {fp} bytes, more than the budget")
                if self.used + fp > self.budget:
                    break
                lane = self._pick_lane(waiting[0].geometry)
                if lane is None:
                    break
                self._admit(waiting.pop(0), now, lane)
            self.max_active = max(self.max_active, len(self.active))
            # groups without a call in flight: launch one with all their active requests
            by_group: dict[tuple, list] = {}
            for r in self.active:
                by_group.setdefault((geometry_key(r.geometry), r._lane), []).append(r)
            for key, reqs in by_group.items():
                if key not in flights:
                    flights[key] = self._launch(self.groups[key], reqs)
                    self.ticks += 1
            # complete whichever calls have finished
            progressed = False
            for key in list(flights):
                if flights[key][3].query():
                    self._complete(self.groups[key], flights.pop(key), clock)
                    progressed = True
            if not progressed:
                if flights:
                    time.sleep(0.0002)
                elif waiting and realtime:
                    time.sleep(max(0.0, min(0.01, waiting[0].arrival - clock())))
        torch.cuda.synchronize(self.device)
        wall = clock()
        lat = np.array([r.latency for r in requests])
        return {"requests": len(requests), "wall_s": wall, "inversions_per_s": len(requests) / wall,
                "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
                "engine_calls": self.engine_calls, "max_active": self.max_active,
                "evaluations": int(sum(r.evaluations for r in requests))}


def batched_prior(part: list, xs):
    """Prior costs and gradients of several requests' unknowns (a list, or an (M, N)
    tensor) at once when they share one prior type and settings, else one by one
    (the requests' unknown counts may then differ; the gradients come back as a list)."""
    p0 = part[0].prior
    if all(type(r.prior) is type(p0) and r.prior.same_settings(p0) for r in part) and \
            hasattr(p0, "batched_cost_and_gradient"):
        return p0.batched_cost_and_gradient(xs if torch.is_tensor(xs) else torch.stack(list(xs)))
    cs, gs = [], []
    for i, r in enumerate(part):
        c, g = r.prior.compute_cost_and_gradient(xs[i][:, None], compute_gradient=True)
        cs.append(c)
        gs.append(g[:, 0])
    return torch.stack(cs), gs


def run_plain(requests: list[InversionRequest], device=None, checkpoint_above_bytes: int | None = None,
              checkpoint_every: int = 50, shots_per_launch: int = 0, engines: dict | None = None) -> dict:
    """One request at a time (one model per engine call), arrivals ignored; a set-up keeps
    whole forward histories when its shots' (or one launch's) fit 60 % of the free device
    memory, else it uses checkpointed adjoints (``checkpoint_above_bytes``: checkpoint
    every set-up above that many whole-history bytes per shot instead).
    ``shots_per_launch=1`` is the plain per-shot form (each shot's sweeps are their own
    launches, one after another)."""
    device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    keep = engines is not None
    engines = {} if engines is None else engines
    t0 = time.perf_counter()
    for r in requests:
        key = geometry_key(r.geometry)
        if key not in engines:
            g = r.geometry
            chunk = shots_per_launch or g.nshots
            engines[key] = Engine(g, max_models=1, max_shots_per_chunk=chunk, device=device)
            if checkpoint_above_bytes is not None:
                ck = shot_workspace_bytes(g, 0) > checkpoint_above_bytes
            else:
                ck = chunk * shot_workspace_bytes(g, 0) > 0.6 * torch.cuda.mem_get_info(device)[0]
            if ck:
                engines[key].set_option("checkpoint_every", checkpoint_every)
        eng = engines[key]
        B = r.prior.basis_vectors
        n = r.geometry.nrecords
        x0 = project(B, r.start.reshape(-1, 1))[:, 0].clone()

        def func(x, r=r, eng=eng, B=B, n=n):
            eng.poll()         # the previous evaluation was read on the host: report its failures
            _, _, grad, mf = eng.vel_to_seis((B @ x[:, None])[:, 0], None, r.target, adjoint_on_residual=True,
                                             want_misfit=True)
            cp, gp = batched_prior([r], x[None, :])     # the server's prior code path, one model
            r.evaluations += 1
            cost, g = (cp[0] + mf[0] / n) * r.scaling, (gp[0] + (2.0 / n) * (B.T @ grad[0])) * r.scaling
            if r.seis_error_tolerance > 0 and float(mf[0]) / n < r.seis_error_tolerance:
                cost, g = 0 * cost, 0 * g
            return cost, g

        x = numerics.bfgs(func, x0, r.maxiter, r.tolerance_grad, r.tolerance_change)
        eng.check()
        r.result = r.start.clone() if torch.isnan(x).any() else (B @ x[:, None])[:, 0]
        r.finished = time.perf_counter() - t0
    torch.cuda.synchronize(device)
    wall = time.perf_counter() - t0
    if not keep:
        for e in engines.values():
            e.close()
    return {"requests": len(requests), "wall_s": wall, "inversions_per_s": len(requests) / wall,
            "evaluations": int(sum(r.evaluations for r in requests))}


def all_shots_workspace(setups: dict, budget: float, checkpoint_every: int) -> dict:
    """Workspace of set-ups that sweep all their shots at once: {key: (geometry, models)} ->
    {key: (checkpoint interval, bytes)}.  Whole histories where ``budget`` bytes allow;
    otherwise the set-ups with the largest history per shot switch to checkpointed adjoints
    first, until the total fits (or every set-up is checkpointed)."""
    ck = {k: 0 for k in setups}
    need = lambda k: setups[k][1] * setups[k][0].nshots * shot_workspace_bytes(setups[k][0], ck[k])
    for k in sorted(setups, key=lambda k: -shot_workspace_bytes(setups[k][0], 0)):
        if sum(need(j) for j in setups) <= budget:
            break
        ck[k] = checkpoint_every
    return {k: (ck[k], need(k)) for k in setups}


def concurrent_workspace(setups: dict, budget: float, checkpoint_every: int, cluster_penalty: float = 3.0) -> dict:
    """Workspace of set-ups whose engines sweep at the same time, each in chunks of shots:
    {key: (geometry, models, fill shots, on clusters)} -> {key: (checkpoint interval, shot slots)}.

    A set-up's chunk must at least fill the GPU on its own (``fill_shots``: one wave of the
    tiled adjoint's resident blocks, or one round of its resident clusters when its adjoint
    runs on clusters), so that its last chunks run at full rate when the other set-ups
    are done.  Whole histories where ``budget`` bytes hold every set-up's minimum chunk;
    otherwise set-ups switch to checkpointed adjoints in order of the most memory freed per
    unit of extra time: the extra time is the recomputed forward, proportional to the
    set-up's point-steps, and ``cluster_penalty`` times that where checkpointing also
    moves the adjoint from its cluster sweep to the tiled one.  Memory left over grows the
    chunks in proportion to each set-up's point-steps (fewer rounds)."""
    shots = {k: m * g.nshots for k, (g, m, _, _) in setups.items()}
    fill = {k: max(1, min(shots[k], f)) for k, (_, _, f, _) in setups.items()}
    work = {k: shots[k] * g.nt * g.padded_shape[0] * g.padded_shape[1] for k, (g, _, _, _) in setups.items()}
    ck = {k: 0 for k in setups}
    per = lambda k: shot_workspace_bytes(setups[k][0], ck[k])
    need = lambda k: fill[k] * per(k)

    def freed_per_time(k):
        g, _, _, c = setups[k]
        saved = fill[k] * (shot_workspace_bytes(g, 0) - shot_workspace_bytes(g, checkpoint_every))
        return saved / (work[k] * (cluster_penalty if c else 1.0))

    while sum(need(k) for k in setups) > budget:
        cand = [k for k in setups if not ck[k]]
        if not cand:
            break
        ck[max(cand, key=freed_per_time)] = checkpoint_every
    spare = max(0.0, budget - sum(need(k) for k in setups))
    total_work = sum(work.values())
    return {k: (ck[k], max(fill[k], min(shots[k], int((need(k) + spare * work[k] / total_work) // per(k)))))
            for k in setups}


def fill_shots(g: Geometry, device) -> tuple[int, bool]:
    """(shots a chunk needs to fill the GPU on its own, whether the adjoint runs on
    clusters), read from a probe engine of the geometry sized for chunks of 64 shots
    (the cluster shape depends on the chunk; the probe allocates no sweep workspace): one
    round of its resident adjoint clusters, or one wave of the tiled adjoint's resident
    blocks (4 per SM)."""
    probe = Engine(g, max_models=64, max_shots_per_chunk=64, device=device)
    try:
        clusters, tiles = int(probe.info("cluster_adj")), int(probe.info("tiles"))
    finally:
        probe.close()
    if clusters:
        return clusters, True
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    return max(1, math.ceil(4 * sms / tiles)), False


class HeterogeneousBatch:
    """Forward + adjoint of models on several grids in one call, one engine per grid.
    Default: each engine's own call on its own stream, all launched before any is waited
    for, so that they overlap (cluster sweeps where a grid has them, graphs of tiled step
    launches elsewhere); the engines share ``memory_fraction`` of the free device memory
    by ``concurrent_workspace``: whole histories where they fit, checkpointed adjoints
    (every ``checkpoint_every`` steps) for the set-ups where that costs the least time.
    ``one_launch``: every grid's sweeps together in one persistent wavefront
    launch per sweep (``seis_vel_to_seis_multi``), each set-up's engine sized to hold all
    its shots at once, checkpointed for the set-ups with the largest history where whole
    histories would not fit (on GB300 about twice the time of the default on the 48-model
    mix: the wavefront forward is slower than the step launches, the 70x70 and 100x140
    set-ups lose their cluster sweeps, and holding every shot at once checkpoints the
    large set-ups).
    Results are bitwise the same either way."""

    def __init__(self, device=None, max_models: int = 64, memory_fraction: float = 0.75,
                 checkpoint_every: int = 50, one_launch: bool = False):
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.max_models = max_models
        self.memory_fraction = memory_fraction
        self.checkpoint_every = checkpoint_every
        self.one_launch = one_launch
        self.groups: dict[tuple, _Group] = {}

    def run(self, jobs: list[tuple]):
        """jobs: (geometry, model vector (nv,), target records (nrecords,)); returns
        [(misfit, gradient)] in job order."""
        by: dict[tuple, list[int]] = {}
        for i, (g, _, _) in enumerate(jobs):
            by.setdefault(geometry_key(g), []).append(i)
        out = [None] * len(jobs)
        pending = []
        new = [k for k in by if k not in self.groups]
        one = self.one_launch and all(len(idx) <= self.max_models for idx in by.values())
        if new and one:
            # one launch per sweep: every set-up holds all its shots at once (one round of chunks)
            free, _ = torch.cuda.mem_get_info(self.device)
            geo = {k: jobs[by[k][0]][0] for k in new}
            plan = all_shots_workspace({k: (geo[k], len(by[k])) for k in new}, self.memory_fraction * free,
                                       self.checkpoint_every)
            for k in new:
                ck, nbytes = plan[k]
                self.groups[k] = _Group(geo[k], self.max_models, ck, self.device, workspace_bytes=nbytes)
        elif new:
            # the new engines share the free device memory by their work (whole histories
            # where chunks that fill the GPU fit)
            free, _ = torch.cuda.mem_get_info(self.device)
            geo = {k: jobs[by[k][0]][0] for k in new}
            plan = concurrent_workspace({k: (geo[k], len(by[k]), *fill_shots(geo[k], self.device)) for k in new},
                                        self.memory_fraction * free, self.checkpoint_every)
            for k in new:
                ck, slots = plan[k]
                self.groups[k] = _Group(geo[k], self.max_models, ck, self.device,
                                        workspace_bytes=slots * shot_workspace_bytes(geo[k], ck))
        if one:
            keys = list(by)
            engines = [self.groups[k].engine for k in keys]
            outs = vel_to_seis_multi(engines, [torch.stack([jobs[i][1] for i in by[k]]) for k in keys],
                                     [torch.stack([jobs[i][2] for i in by[k]]) for k in keys],
                                     adjoint_on_residual=True, want_misfit=True)
            torch.cuda.current_stream(self.device).synchronize()
            for k, (_, gr, mf), eng in zip(keys, outs, engines):
                eng.poll()
                for j, i in enumerate(by[k]):
                    out[i] = (mf[j], gr[j])
            return out
        for key, idx in by.items():
            grp = self.groups[key]
            # geometries of this run overlap on the device: side sweeps only for a lone one
            for opt in ("fwd_side", "adj_side"):
                grp.engine.set_option(opt, 0 if len(by) > 1 else -1)
            grp.stream.wait_stream(torch.cuda.current_stream(self.device))
            for i0 in range(0, len(idx), self.max_models):
                part = idx[i0:i0 + self.max_models]
                with torch.cuda.stream(grp.stream):
                    v = torch.stack([jobs[i][1] for i in part])
                    t = torch.stack([jobs[i][2] for i in part])
                    _, _, gr, mf = grp.engine.vel_to_seis(v, None, t, adjoint_on_residual=True, want_misfit=True,
                                                          stream=grp.stream)
                pending.append((grp, part, gr, mf))
        for grp, part, gr, mf in pending:
            grp.stream.synchronize()
            grp.engine.poll()
            for j, i in enumerate(part):
                out[i] = (mf[j], gr[j])
        return out
