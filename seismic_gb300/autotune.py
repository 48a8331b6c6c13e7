"""Launch-configuration autotuner of the engine.

For one workload (geometry, models per call) it times the candidate
configurations of the engine on seeded synthetic models -- sweep path (tiled
sweeps or cluster-resident sweeps), the time steps fused per launch (the
cluster sweeps fuse all nt; the tiled ones one or two), forward cluster shape
(8, 10 or 16 CTAs, i.e. 40-, 32- or 20-row bands), adjoint cluster shape (10
CTAs with tensor-memory state, or 16), grid columns per thread of the cluster
sweeps (1 or 2), and how many shots sweep concurrently -- and keeps the
fastest.  A second stage times the side sweeps of the winner: how many of a
chunk's shots run beside the cluster sweeps on the SMs the clusters leave free,
on the tiled kernels or (the forward beside 10-CTA clusters) on two 8-CTA cluster
sweeps (the engine's own split comes from measured throughputs; the tuner tries
it, none, and the splits that give the main clusters up to four rounds fewer).  Results are cached in a JSON file keyed by
the device name, the geometry and the batch size, so a service tunes each
workload once.

    cfg = autotune.tune(geometry, nmodels=64)
    engine = autotune.tuned_engine(geometry, nmodels=64)
"""
from __future__ import annotations

import json
import os
import time

import numpy as np
import torch

from . import synthetic
from .engine import Engine
from .geometry import Geometry

DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_tuning", "engine_configs.json")


def _key(geometry: Geometry, nmodels: int, gradient: bool) -> str:
    g = geometry
    dev = torch.cuda.get_device_name()
    return (f"{dev}|{g.nz}x{g.nx}|nbc{g.nbc}|nt{g.nt}|shots{g.nshots}|rec{g.nrec}|dt{g.dt}|dx{g.dx}|f{g.freq}|"
            f"models{nmodels}|grad{int(gradient)}")


def candidates(geometry: Geometry, nmodels: int) -> list[dict]:
    """Configurations worth timing for this workload."""
    shots = nmodels * geometry.nshots
    chunks = sorted({0, geometry.nshots, min(shots, 96)} | ({shots} if shots > 1 else set()))
    out = []
    for chunk in chunks:
        for fuse in (1, 0):
            out.append({"sweep_path": 1, "fuse": fuse, "fwd_cluster": 8, "columns": 2, "chunk": chunk})
        for fc in (8, 10, 16):
            for cols in (2, 1):
                for ac in ((10, 16) if cols == 2 else (16,)):
                    out.append({"sweep_path": 2, "fwd_cluster": fc, "columns": cols, "adj_cluster": ac,
                                "chunk": chunk})
    return out


def side_candidates(eng: Engine, cfg: dict) -> list[dict]:
    """Side-sweep splits to time for a cluster configuration (whose first-stage timing is
    the engine's own split): none (0), and the splits that leave the clusters 0..3 rounds
    fewer than all slots need -- for the forward both on the tiled kernels and, beside
    10-CTA clusters, on two concurrent 8-CTA cluster sweeps."""
    if cfg["sweep_path"] != 2:
        return []
    S = eng.slots
    out = []
    fwd_ncl = eng.info({8: "cluster_fwd", 10: "cluster_fwd10", 16: "cluster_fwd16"}[cfg["fwd_cluster"]])
    for key, ncl, extra in (("adj_side", eng.info("cluster_adj"), [{}]),
                            ("fwd_side", fwd_ncl, [{"fwd_side_cluster": 0}] +
                             ([{"fwd_side_cluster": 8}] if cfg["fwd_cluster"] == 10 else []))):
        if ncl < 1 or S < 2 * ncl:
            continue
        rounds = -(-S // ncl)
        sides = {0} | {S - r * ncl for r in range(max(1, rounds - 4), rounds + 1) if 0 < S - r * ncl < S}
        out += [dict(cfg, **{key: n}, **x) for x in extra for n in sorted(sides)]
    return out


def _apply(eng: Engine, cfg: dict) -> bool:
    try:
        eng.set_option("sweep_path", cfg["sweep_path"])
        eng.set_option("fwd_fuse", cfg.get("fuse", 1))
        eng.set_option("adj_fuse", cfg.get("fuse", 1))
        if cfg["sweep_path"] == 2:
            eng.set_option("fwd_cluster", cfg["fwd_cluster"])
            eng.set_option("columns", cfg.get("columns", 2))
            if eng.info("fwd_columns") != cfg.get("columns", 2):
                return False                    # column pairs do not apply (odd padded width)
            if cfg.get("adj_cluster"):
                eng.set_option("adj_cluster", cfg["adj_cluster"])
            for key in ("adj_side", "fwd_side", "fwd_side_cluster"):
                if key in cfg:
                    eng.set_option(key, cfg[key])
        return True
    except Exception:
        return False        # the configuration does not apply to this geometry


def time_config(geometry: Geometry, nmodels: int, cfg: dict, gradient: bool = True, repeats: int = 2,
                seed: int = 0) -> float | None:
    """Median seconds of one call (cost + gradient, or forward only) with ``cfg``; None if
    the configuration does not apply."""
    vecs, trues, _ = synthetic.batch(seed, nmodels, geometry.nz, geometry.nx)
    eng = Engine(geometry, max_models=nmodels, max_shots_per_chunk=cfg["chunk"])
    try:
        if not _apply(eng, cfg):
            return None
        v = torch.as_tensor(vecs, device="cuda")
        t = eng.vel_to_seis(torch.as_tensor(trues, device="cuda"))[0] if gradient else None
        call = (lambda: eng.vel_to_seis(v, None, t, adjoint_on_residual=True)) if gradient else \
            (lambda: eng.vel_to_seis(v))
        call()
        torch.cuda.synchronize()
        times = []
        for _ in range(repeats):
            t0 = time.perf_counter()
            call()
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        return float(np.median(times))
    finally:
        eng.close()


def tune(geometry: Geometry, nmodels: int, gradient: bool = True, cache_path: str = DEFAULT_CACHE,
         refresh: bool = False, cands: list[dict] | None = None) -> dict:
    """Best configuration for the workload (from the cache unless ``refresh``)."""
    key = _key(geometry, nmodels, gradient)
    cache = {}
    if os.path.exists(cache_path):
        with open(cache_path) as f:
            cache = json.load(f)
    if key in cache and not refresh:
        return cache[key]
    results = []
    for cfg in (cands or candidates(geometry, nmodels)):
        t = time_config(geometry, nmodels, cfg, gradient)
        if t is not None:
            results.append((t, cfg))
    if not results:
        raise RuntimeError("no engine configuration applies to this geometry")
    t_best, best = min(results, key=lambda r: r[0])
    if cands is None and best["sweep_path"] == 2:
        # second stage: the side sweeps of the winning cluster configuration
        eng = Engine(geometry, max_models=nmodels, max_shots_per_chunk=best["chunk"])
        try:
            side = side_candidates(eng, best) if _apply(eng, best) else []
        finally:
            eng.close()
        for cfg in side:
            t = time_config(geometry, nmodels, cfg, gradient)
            if t is not None:
                results.append((t, cfg))
        t_best, best = min(results, key=lambda r: r[0])
    entry = dict(best, seconds=t_best, timings=[dict(c, seconds=t) for t, c in results])
    cache[key] = entry
    os.makedirs(os.path.dirname(cache_path), exist_ok=True)
    tmp = cache_path + f".{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1)
    os.replace(tmp, cache_path)
    return entry


def tuned_engine(geometry: Geometry, nmodels: int, gradient: bool = True, cache_path: str = DEFAULT_CACHE) -> Engine:
    """An engine configured with the tuned choice for this workload."""
    cfg = tune(geometry, nmodels, gradient, cache_path)
    eng = Engine(geometry, max_models=nmodels, max_shots_per_chunk=cfg["chunk"])
    _apply(eng, cfg)
    return eng
