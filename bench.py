#!/usr/bin/env python
"""Benchmark of the batched FWI cost + gradient evaluation on GB300.

Workload (one "step"): the misfit and its gradient for 64 seeded 70x70 models
(layered / faulted / curved, 1500-4500 m/s) x 5 shots, nt = 1000, dt = 1 ms,
15 Hz Ricker, 70 surface receivers, i.e. one forward sweep and one adjoint
sweep of 320 shots -- the reference's vel_to_seis(vec, vec_adjoint=target,
adjoint_on_residual=True) (core/seis_forward2.py:146) for 64 models at once.
Targets are the records of +-5% smoothed perturbations of the models.

Metric: shot-steps/s, one shot-step = one shot advanced one time step in one
sweep (forward or adjoint), as the reference's recorded 9,990 shot-steps per
evaluation counts them.  ``value`` is device-resident throughput; ``e2e`` is
the same through the engine API with the step's inputs copied from pinned host
memory and the gradient + misfit copied back inside the timed region.

--impl reference times the reference algorithm on the host cores (the FP64 C
restatement in oracle/, all threads, a bounded sample per step).

Multi-GPU (torchrun): every rank runs its own 64 models (replicas, weak
scaling, no data-path collective); value = all ranks' shot-steps / max time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NZ = NX = 70
NSHOTS = 5
NT = 1000
NMODELS = 64
FWD_BYTES = 16   # algorithmic FP32 bytes per forward point-step: read p, u, alpha; write p (+u)
ADJ_BYTES = 24   # per adjoint point-step: read lambda, mu, alpha, u_{t+1}, u_{t+2}; write lambda


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--models", type=int, default=NMODELS)
    ap.add_argument("--chunk", type=int, default=0, help="shots swept concurrently (0 = engine default)")
    ap.add_argument("--cpu-sample-models", type=int, default=0, help="models per CPU-baseline sample (0 = cores)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", action="store_true",
                    help="small-case mode for ncu: set-up, --warmup calls and one more call, no timing report")
    ap.add_argument("--nt", type=int, default=NT, help="time steps (profiling cases only; the benchmark uses 1000)")
    ap.add_argument("--profile-sweep", choices=["gradient", "tangent"], default="gradient",
                    help="profiling cases only: cost+gradient calls, or forward+tangent calls (J v)")
    ap.add_argument("--fwd-cluster", type=int, default=0, choices=[0, 8, 10, 16],
                    help="CTAs per forward cluster (0 = engine default)")
    ap.add_argument("--adj-side", type=int, default=-1,
                    help="slots per chunk whose adjoint runs tiled beside the clusters (-1 = engine default)")
    ap.add_argument("--fwd-side", type=int, default=-1,
                    help="slots per chunk whose forward runs tiled beside the clusters (-1 = engine default)")
    ap.add_argument("--columns", type=int, default=0, choices=[0, 1, 2],
                    help="grid columns per thread of the cluster sweeps (0 = engine default)")
    ap.add_argument("--tuned", action="store_true",
                    help="batched: use the autotuner's configuration for the workload (tunes it on first use)")
    ap.add_argument("--fwd-tmem", type=int, default=-1, choices=[-1, 0, 1],
                    help="cluster forward: alpha in tensor memory (1) or shared memory (0); -1 = engine default")
    ap.add_argument("--adj-cluster", type=int, default=0, choices=[0, 10, 16],
                    help="CTAs per cluster of the cluster adjoint (0 = engine default)")
    ap.add_argument("--adj-rows", type=int, default=0, choices=[0, 8, 11],
                    help="rows per thread of the tensor-memory adjoint (0 = engine default)")
    ap.add_argument("--neighbour-shuffle", type=int, default=0, choices=[0, 1],
                    help="cluster forward: horizontal neighbours by warp shuffles (1) or shared loads (0)")
    ap.add_argument("--one-step", action="store_true",
                    help="tiled sweeps: one time step per launch (no two-step kernels)")
    ap.add_argument("--path", choices=["auto", "tiled", "wave"], default="auto",
                    help="profiling cases only: force the tiled per-step sweeps, or the tiled kernels "
                         "as one persistent wavefront launch per sweep")
    ap.add_argument("--mode", choices=["batched", "serve", "hetero", "gn", "wave"], default="batched",
                    help="batched: the benchmark line; serve: continuous batching of whole inversions vs one at "
                         "a time; hetero: one call over models on different grids and nt; gn: batched "
                         "Gauss-Newton-CG (fused matvecs) on 70x70 and 200x300 models vs the two-call form")
    ap.add_argument("--gn-iters", type=int, default=10, help="gn: Gauss-Newton iterations (CG 20 matvecs each)")
    ap.add_argument("--gn-models", type=int, default=8, help="gn: models per grid")
    ap.add_argument("--requests", type=int, default=32, help="serve: number of requests")
    ap.add_argument("--lanes", type=int, default=2, help="serve: engines (lanes) of the homogeneous server")
    ap.add_argument("--maxiter", type=int, default=10, help="serve: L-BFGS iterations per request")
    ap.add_argument("--rate", type=float, default=20.0, help="serve: Poisson arrival rate (requests/s)")
    ap.add_argument("--no-serve", action="store_true",
                    help="batched: skip the served-vs-plain inversion leg of the benchmark line")
    ap.add_argument("--serve-inversions", type=int, default=64,
                    help="batched: inversions of the served-vs-plain leg (L-BFGS(--maxiter) + TV, 70x70)")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def workload(seed, nmodels, eng_factory=None):
    from seismic_gb300 import synthetic
    vecs, trues, fams = synthetic.batch(seed, nmodels, NZ, NX)
    return vecs, trues, fams


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_profile(kernel):
    """Per-point-step figures of ``kernel`` from its committed ncu summary
    (``profiles/<kernel>__*.md``: lines ``name: value``), with the file's name."""
    import glob
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", f"{kernel}__*.md"))):
        vals = {}
        with open(path) as f:
            for line in f:
                if ":" in line and line.split(":", 1)[0].endswith(("_per_point_step", "_pipe_active")):
                    try:
                        vals[line.split(":", 1)[0].strip()] = float(line.split(":", 1)[1].split()[0])
                    except ValueError:
                        pass
        if vals:
            vals["file"] = os.path.relpath(path, ROOT)
            return vals
    return {}


SMEM_WAVEFRONT_BYTES = 128   # one shared-memory wavefront per clock per SM is the LSU pipe's peak


def kernel_roofline(kern, point_steps, bytes_per_launch, avg_launch_s, clocks, nsm, busy_sms):
    """Roofline object of the dominant sweep kernel.  Cluster kernels keep the wavefields
    in shared memory, so their bound is the shared-memory pipe: achieved = shared-memory
    wavefronts per point-step (from the kernel's ncu summary) x 128 B x point-steps / the
    launch time measured here; peak = 128 B per clock per SM x SMs x the median SM clock
    sampled during the timed region.  Their algorithmic-byte figure (which exceeds the HBM
    peak, the fields being on chip) is kept as ``effective_hbm``; their real DRAM traffic
    is the history stream (``traffic``, ``dram_gbs``).  Tiled kernels stream their fields
    through HBM: bound hbm, achieved = algorithmic bytes / time."""
    hbm_peak, peak_kind = load_peaks()
    prof = load_profile(kern)
    eff = bytes_per_launch / avg_launch_s / 1e9
    traffic = prof["dram_bytes_per_point_step"] * point_steps if "dram_bytes_per_point_step" in prof else None
    common = {"kernel": kern, "traffic": traffic, "bytes_per_launch": bytes_per_launch,
              "avg_launch_us": avg_launch_s * 1e6, "point_steps_per_launch": point_steps,
              "profile": prof.get("file")}
    if "cluster" not in kern:
        return {"bound": "hbm", "achieved": eff, "peak": hbm_peak, "unit": "GB/s", "frac": eff / hbm_peak,
                "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)", **common}
    sm_mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    peak = SMEM_WAVEFRONT_BYTES * nsm * sm_mhz * 1e6 / 1e9
    wf = prof.get("smem_wavefronts_per_point_step")
    achieved = wf * SMEM_WAVEFRONT_BYTES * point_steps / avg_launch_s / 1e9 if wf else None
    out = {"bound": "smem", "achieved": achieved, "peak": peak, "unit": "GB/s",
           "frac": achieved / peak if achieved else None,
           "peak_kind": f"derived: {SMEM_WAVEFRONT_BYTES} B/clock/SM x {nsm} SMs x {sm_mhz:.0f} MHz (median under load)",
           "busy_sms": busy_sms, **common}
    if achieved and busy_sms:
        out["frac_on_busy_sms"] = achieved / peak * nsm / busy_sms
    if traffic is not None:
        out["dram_gbs"] = traffic / avg_launch_s / 1e9
        out["dram_frac"] = out["dram_gbs"] / hbm_peak
    if "fma_pipe_active" in prof:
        out["fp32_issue_frac"] = prof["fma_pipe_active"]     # FMA pipe active, from the ncu summary
    out["effective_hbm"] = {"achieved": eff, "peak": hbm_peak, "frac": eff / hbm_peak,
                            "what": "algorithmic FP32 bytes (forward 16, adjoint 24 per point-step) / launch time; "
                                    "above 1 because the wavefields stay in shared memory"}
    return out


def serve_leg(n, maxiter):
    """Whole inversions served with continuous batching against the plain form: n
    L-BFGS(maxiter) + TV inversions of 70x70 / 5-shot / nt=1000 models from smoothed
    starts, all arriving at once; served = two lanes sharing one engine (each call with
    the whole GPU), plain = one request at a time, one shot per launch.  Results must be
    bitwise the same."""
    import torch

    from seismic_gb300.geometry import Geometry
    from seismic_gb300.serving import InversionServer, run_plain
    torch.cuda.empty_cache()
    free, _ = torch.cuda.mem_get_info()
    fwd = {}
    g70 = [Geometry.surface(70, 70, 5, NT)]
    server = InversionServer(hbm_budget_bytes=int(0.5 * free), max_batch=max(1, n // 2), max_geometries=1, lanes=2)
    server.run(_serve_requests([0] * n, [0.0] * n, g70, 1, fwd), realtime=False)      # warm-up
    served = _serve_requests([0] * n, [0.0] * n, g70, maxiter, fwd)
    sa = server.run(served, realtime=False)
    server.close()
    plain_engines = {}
    run_plain(_serve_requests([0], [0.0], g70, 1, fwd), shots_per_launch=1, engines=plain_engines)
    plain = _serve_requests([0] * n, [0.0] * n, g70, maxiter, fwd)
    pa = run_plain(plain, shots_per_launch=1, engines=plain_engines)
    # the same inversions with the optimiser resident on the GPU: one batched engine call
    # and one optimiser launch per evaluation, no host read per evaluation
    from seismic_gb300 import inversion
    from seismic_gb300.engine import Engine
    dev = _serve_requests([0] * n, [0.0] * n, g70, maxiter, fwd)
    eng = Engine(g70[0], max_models=n)
    tg = torch.stack([r.target for r in dev])
    st = torch.stack([r.start for r in dev])
    inversion.seis_to_vel_lbfgs_batched(tg, st, dev[0].prior, eng, maxiter=1)       # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out_dev, dev_evals = inversion.seis_to_vel_lbfgs_batched(tg, st, dev[0].prior, eng, maxiter=maxiter)
    torch.cuda.synchronize()
    dev_wall = time.perf_counter() - t0
    eng.close()
    for e in list(plain_engines.values()) + list(fwd.values()):
        e.close()
    same = all(torch.equal(a.result, b.result) for a, b in zip(served, plain))
    dmod = max(float((out_dev[i] - served[i].result).abs().max() / served[i].result.abs().max()) for i in range(n))
    what = f"{n} x L-BFGS({maxiter}) + TV, 70x70, 5 shots, nt={NT}, smoothed starts, all arriving at t=0"
    return {"served": {"inversions_per_s": sa["inversions_per_s"], "p50_latency_s": sa["p50_latency_s"],
                       "p99_latency_s": sa["p99_latency_s"], "wall_s": sa["wall_s"], "evaluations": sa["evaluations"],
                       "engine_calls": sa["engine_calls"], "speedup_vs_plain": sa["inversions_per_s"] /
                       pa["inversions_per_s"], "results_identical_to_plain": same, "what": what},
            "plain_served": {"inversions_per_s": pa["inversions_per_s"], "wall_s": pa["wall_s"],
                             "evaluations": pa["evaluations"],
                             "what": "the same requests one at a time, one shot per launch"},
            "device_loop": {"inversions_per_s": n / dev_wall, "wall_s": dev_wall, "evaluation_rounds": dev_evals,
                            "max_model_rel_diff_vs_served": dmod,
                            "what": "the same inversions, all models per engine call, L-BFGS on the GPU "
                                    "(fixed-order reductions: not bitwise the served run's torch reductions)"}}


def cpu_baseline(nmodels_sample, threads, forward=False):
    """The oracle (FP64 C restatement of the reference) on host cores: one
    cost+gradient evaluation of `nmodels_sample` models, one model per thread
    (``forward``: also their forward-only evaluation; returns its rate and time too)."""
    from oracle import oracle
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=NT)
    vecs, trues, _ = workload(4242, nmodels_sample)
    t0 = time.perf_counter()
    targets = oracle.batch_forward(g, trues, threads)
    dt_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    oracle.batch_cost_gradient(g, vecs, targets, threads)
    dt = time.perf_counter() - t0
    shot_steps = nmodels_sample * NSHOTS * NT * 2
    if forward:
        return shot_steps / dt, dt, shot_steps / 2 / dt_fwd, dt_fwd
    return shot_steps / dt, dt


def run_reference(args, world, rank):
    """The reference's algorithm on the host cores: the FP64 oracle, one model per thread.
    Each step is a bounded sample of the benchmark workload (``--cpu-sample-models``
    models, default one per core) so that the run ends within minutes; the rate is
    per shot-step, the same unit as the GPU arm.  ``ms_per_step`` is the measured time
    of one sample step (not scaled to the 64 models of the workload)."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = args.cpu_sample_models or threads
    vals, secs = [], []
    for i in range(args.warmup + args.steps):
        v, dt = cpu_baseline(n, threads)
        if i >= args.warmup:
            vals.append(v)
            secs.append(dt)
    value = statistics.median(vals)
    sample = (f"{n} of the workload's {NMODELS} models per step ({n} x {NSHOTS} shots x {NT} steps, forward + "
              f"adjoint), one model per thread")
    out = {
        "impl": "reference", "metric": "shot_steps_per_s", "value": value, "unit": "shot-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * statistics.median(secs), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(NMODELS, world),
        "sample": {"models_per_step": n, "shot_steps_per_step": n * NSHOTS * NT * 2, "what": sample},
        "cpu_baseline": {"value": value, "unit": "shot-steps/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "shot-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def bench_config(nm, world):
    """The workload as both arms name it."""
    return {"workload": f"cost+gradient, {nm} models x {NSHOTS} shots, 70x70 (310x310 padded), nt={NT}",
            "models": nm, "grid": [NZ, NX], "nshots": NSHOTS, "nt": NT,
            "l2": "working set > L2 (forward increment history ~0.4 GB per shot)",
            "parallelism": f"replicas x{world}"}


def run_ours(args, world, rank, local):
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())
    from seismic_gb300.engine import Engine
    from seismic_gb300.geometry import Geometry

    g = Geometry.reference(nt=args.nt if args.profile else NT)
    nm = args.models
    vecs_np, trues_np, fams = workload(1000 + rank, nm)
    if args.tuned:
        # the autotuner's choice for this workload (timed on first use, then cached)
        from seismic_gb300 import autotune
        eng = autotune.tuned_engine(g, nm)
    else:
        eng = Engine(g, max_models=nm, max_shots_per_chunk=args.chunk)
    if args.profile and args.path != "auto":
        eng.set_option("sweep_path", {"tiled": 1, "wave": 3}[args.path])
    if args.fwd_cluster:
        eng.set_option("fwd_cluster", args.fwd_cluster)
    if args.adj_side != -1:
        eng.set_option("adj_side", args.adj_side)
    if args.fwd_side != -1:
        eng.set_option("fwd_side", args.fwd_side)
    if args.columns:
        eng.set_option("columns", args.columns)
    if args.neighbour_shuffle:
        eng.set_option("neighbour_shuffle", 1)
    if args.fwd_tmem >= 0:
        eng.set_option("fwd_tmem", args.fwd_tmem)
    if args.adj_cluster:
        eng.set_option("adj_cluster", args.adj_cluster)
    if args.adj_rows:
        eng.set_option("adj_rows", args.adj_rows)
    if args.one_step:
        eng.set_option("fwd_fuse", 0)
        eng.set_option("adj_fuse", 0)
    vecs = torch.as_tensor(vecs_np, device=dev)
    trues = torch.as_tensor(trues_np, device=dev)
    targets, _, _, _ = eng.vel_to_seis(trues)          # observed data (untimed)
    torch.cuda.synchronize()
    if args.profile:
        dirs = torch.as_tensor(np.random.default_rng(7).normal(0.0, 5.0, vecs_np.shape), device=dev)
        for _ in range(args.warmup + 1):
            if args.profile_sweep == "tangent":
                eng.vel_to_seis(vecs, dirs)
            else:
                eng.vel_to_seis(vecs, None, targets, adjoint_on_residual=True, want_misfit=True)
        st = eng.stats()
        print(json.dumps({"profile": True, "models": nm, "nt": g.nt, "slots": eng.slots, **st}))
        return

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    stream = torch.cuda.current_stream(dev)
    step = lambda: eng.vel_to_seis(vecs, None, targets, adjoint_on_residual=True, want_misfit=True)
    for _ in range(args.warmup):
        step()
    barrier()
    launches0 = eng.stats()["launches"]
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(dev.index) as clk:
        barrier()
        t0 = time.perf_counter()
        for i in range(args.steps):
            evs[i][0].record(stream)
            _, _, grad, mf = step()
            evs[i][1].record(stream)
        barrier()
        wall = time.perf_counter() - t0
    st = eng.stats()
    last = {k: eng.info(k) for k in ("last_fwd_path", "last_adj_path", "last_fwd_launches", "last_adj_launches",
                                     "last_adj_side", "last_fwd_side", "last_adj_cluster_ns")}
    launches = st["launches"] - launches0
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    shot_steps_rank = nm * NSHOTS * NT * 2
    value = world * shot_steps_rank * args.steps / (total_ms / 1000.0)

    # end to end through the engine API with HOST buffers: the call uploads the models
    # and targets itself (the targets while the forward sweep runs) and returns the
    # records, gradient and misfit in pinned host memory (the records while the adjoint
    # sweep runs); it returns once they are complete
    vec_h = torch.as_tensor(vecs_np).pin_memory()
    tgt_h = targets.cpu().pin_memory()
    outs = {}

    def e2e_step():
        res, _, gr, m = eng.vel_to_seis(vec_h, None, tgt_h, adjoint_on_residual=True, want_misfit=True)
        outs.update(res=res, grad=gr, mf=m)

    # W untimed warm-up calls, as for the device-resident steps: the first two calls also
    # fill the host allocator's cache of pinned output buffers (a call's outputs are still
    # held while the next one allocates its own)
    for _ in range(max(2, args.warmup)):
        e2e_step()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    if world > 1:
        t = torch.tensor([e2e_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_value = world * shot_steps_rank * args.steps / (e2e_ms / 1000.0)
    h2d = vec_h.numel() * 8 + tgt_h.numel() * 8
    d2h = sum(outs[k].numel() * 8 for k in ("res", "grad", "mf"))
    assert all(outs[k].device.type == "cpu" for k in outs)

    # plain form: one shot per launch (one model per call, its shots swept one at a time)
    plain = Engine(g, max_models=1, max_shots_per_chunk=1)
    pv, pt = vecs[:1].clone(), targets[:1].clone()
    for _ in range(3):
        plain.vel_to_seis(pv, None, pt, adjoint_on_residual=True)
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nplain = 8
    p0.record(stream)
    for _ in range(nplain):
        plain.vel_to_seis(pv, None, pt, adjoint_on_residual=True)
    p1.record(stream)
    torch.cuda.synchronize()
    plain_ms = p0.elapsed_time(p1) / nplain
    plain.close()

    # roofline of the dominant sweep kernel (last timed call's sweeps); a launch of
    # the cluster kernels runs a whole chunk's sweep, a tiled launch one time step
    npad = g.padded_shape[0] * g.padded_shape[1]
    shots = nm * NSHOTS
    fwd_ms, adj_ms = st["fwd_ms"], st["adj_ms"]
    # (the tiled sweeps of this even-width grid take two steps per launch)
    names = {("fwd", 1): "fwd_step2_kernel", ("fwd", 2): "fwd_cluster_tm_kernel" if eng.info("fwd_tmem") else "fwd_cluster_kernel",
             ("adj", 1): "adj_step2_kernel", ("adj", 2): "adj_cluster_kernel"}
    nchunks = -(-shots // eng.slots)
    busy_sms = None
    if adj_ms >= fwd_ms and last["last_adj_path"] == 2:
        # cluster adjoint: one launch per chunk over the slots not given to the side
        # adjoint (which runs beside it on the SMs the clusters leave free), timed
        # with events around the cluster launches themselves
        kern, bpp = ("adj_cluster_tm_kernel" if eng.info("adj_tmem") else names[("adj", 2)]), ADJ_BYTES
        nl = nchunks
        bytes_per_launch = bpp * npad * (shots - last["last_adj_side"]) * NT / nl
        avg_launch_s = last["last_adj_cluster_ns"] / 1e9 / nl
        busy_sms = eng.info("cluster_adj") * eng.info("adj_cluster")
    else:
        if adj_ms >= fwd_ms:
            kern, bpp, sweep_ms = names[("adj", last["last_adj_path"])], ADJ_BYTES, adj_ms
            nl = last["last_adj_launches"]
        else:
            kern, bpp, sweep_ms = names[("fwd", last["last_fwd_path"])], FWD_BYTES, fwd_ms
            nl = last["last_fwd_launches"]
            if last["last_fwd_path"] == 2:
                fc = eng.info("fwd_cluster")
                busy_sms = eng.info({8: "cluster_fwd", 10: "cluster_fwd10", 16: "cluster_fwd16"}[fc]) * fc
        bytes_per_launch = bpp * npad * shots * NT / nl
        avg_launch_s = sweep_ms / 1000.0 / nl
    point_steps = bytes_per_launch / bpp
    roofline = kernel_roofline(kern, point_steps, bytes_per_launch, avg_launch_s, clk.summary(),
                               torch.cuda.get_device_properties(dev).multi_processor_count, busy_sms)

    out = {
        "metric": "shot_steps_per_s", "value": value, "unit": "shot-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded layered/faulted/curved 70x70 models; targets from 5% perturbed copies)",
        "config": bench_config(nm, world),
        "engine": {"chunk_shots": eng.slots, "fwd_cluster": eng.info("fwd_cluster"), "tuned": bool(args.tuned),
                   "fwd_neighbour_shuffle": eng.info("fwd_shuffle"), "fwd_tensor_memory": eng.info("fwd_tmem"),
                   "adj_cluster": eng.info("adj_cluster"),
                   "adj_tensor_memory": eng.info("adj_tmem"),
                   "adj_side_slots": last["last_adj_side"], "fwd_side_slots": last["last_fwd_side"],
                   "fwd_side_cluster": eng.info("fwd_side_cluster"),
                   "fwd_sweep_ms": fwd_ms, "adj_sweep_ms": adj_ms},
        "e2e": {"value": e2e_value, "unit": "shot-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "evals_per_s": world * nm * args.steps / (total_ms / 1000.0),
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99)),
                       "what": f"one {nm}-model cost+gradient step"},
        "plain": {"value": NSHOTS * NT * 2 / (plain_ms / 1000.0), "unit": "shot-steps/s",
                  "ms_per_eval": plain_ms, "what": "1 model x 5 shots per call, one shot per launch"},
        "roofline": roofline,
        "clocks": clk.summary(),
        "wall_s": wall,
    }
    eng.close()
    if rank == 0 and world == 1 and not args.no_serve:
        out.update(serve_leg(args.serve_inversions, args.maxiter))
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        n = args.cpu_sample_models or threads
        v, dt, vf, dtf = cpu_baseline(n, threads, forward=True)
        # one model per thread at a time: each thread ran ceil(n / threads) 5-shot evaluations
        per_eval = dt / -(-n // threads)
        evals = out.get("served", {}).get("evaluations", 0) / max(1, args.serve_inversions) or 12.0
        out["cpu_baseline"] = {"value": v, "unit": "shot-steps/s", "cores": threads, "kind": "port",
                               "sample": f"{n} models x {NSHOTS} shots x {NT} steps fwd+adj ({dt:.1f} s), "
                                         f"one model per thread",
                               "forward_only": {"value": vf, "unit": "shot-steps/s", "s": dtf},
                               "s_per_evaluation_one_core": per_eval,
                               "inversions_per_s_extrapolated": {
                                   "value": threads / (evals * per_eval), "evaluations_per_inversion": evals,
                                   "what": "L-BFGS(10)+TV inversions on all cores at the served run's mean "
                                           "evaluation count"}}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


SERVE_MIX = [  # (share, nz, nx, shots, nt): the request grids and acquisition set-ups of the stream
    (0.35, 70, 70, 5, 1000), (0.35, 70, 70, 10, 1500), (0.20, 200, 300, 10, 1500), (0.10, 350, 500, 20, 2000)]


def _serve_requests(kinds, arrivals, geoms, maxiter, fwd_engines):
    """One inversion request per entry; request i's models come from seed 5000+i, so the
    same list can be rebuilt for the one-at-a-time run."""
    import torch

    from seismic_gb300 import priors, synthetic
    from seismic_gb300.engine import Engine
    from seismic_gb300.serving import InversionRequest
    reqs = []
    for i, (k, arr) in enumerate(zip(kinds, arrivals)):
        g = geoms[k]
        if k not in fwd_engines:
            fwd_engines[k] = Engine(g, max_models=1, max_shots_per_chunk=g.nshots)
        rng = np.random.default_rng(5000 + i)
        vt = synthetic.model(rng, ["layered", "faulted", "curved"][i % 3], g.nz, g.nx)
        v0 = synthetic.smoothed(vt, 4.0)
        tgt = fwd_engines[k].vel_to_seis(torch.as_tensor(synthetic.to_vector(vt), device="cuda"))[0][0]
        pr = priors.TotalVariation(g.nz, g.nx, device="cuda")
        pr.lam = 1e-6
        pr.prep()
        reqs.append(InversionRequest(rid=i, geometry=g, target=tgt, prior=pr, maxiter=maxiter, arrival=float(arr),
                                     start=torch.as_tensor(synthetic.to_vector(v0, vt.min()), device="cuda")))
    return reqs


def run_serve(args):
    """(a) the spec comparison: 64 whole inversions of 70x70 / 5-shot / nt=1000
    models served with continuous batching vs the plain form (one request at a time,
    one shot per launch); (b) a Poisson stream over the grid mix, p50/p99 latency."""
    import torch

    from seismic_gb300.geometry import Geometry
    from seismic_gb300.serving import InversionServer, run_plain
    torch.cuda.set_device(0)
    free, _ = torch.cuda.mem_get_info()
    fwd = {}
    # (a) homogeneous 70x70 / 5 shots / nt=1000
    g70 = [Geometry.surface(70, 70, 5, NT)]
    nh = 64
    server = InversionServer(hbm_budget_bytes=int(0.5 * free), max_batch=nh // args.lanes, max_geometries=1,
                             lanes=args.lanes)
    # warm-up: the server's engine allocates its workspace and loads its kernels once
    server.run(_serve_requests([0] * nh, [0.0] * nh, g70, 1, fwd), realtime=False)
    served = _serve_requests([0] * nh, [0.0] * nh, g70, args.maxiter, fwd)
    sa = server.run(served, realtime=False)
    server.close()
    plain_engines = {}
    run_plain(_serve_requests([0], [0.0], g70, 1, fwd), shots_per_launch=1, engines=plain_engines)
    plain = _serve_requests([0] * nh, [0.0] * nh, g70, args.maxiter, fwd)
    pa = run_plain(plain, shots_per_launch=1, engines=plain_engines)
    for e in plain_engines.values():
        e.close()
    same_a = all(torch.equal(a.result, b.result) for a, b in zip(served, plain))
    # (b) Poisson stream over the grid mix
    rng = np.random.default_rng(2024)
    shares = np.array([m[0] for m in SERVE_MIX])
    geoms = [Geometry.surface(nz, nx, ns, nt) for _, nz, nx, ns, nt in SERVE_MIX]
    kinds = [int(k) for k in rng.choice(len(SERVE_MIX), size=args.requests, p=shares / shares.sum())]
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, args.requests))
    mixed = _serve_requests(kinds, arrivals, geoms, args.maxiter, fwd)
    server = InversionServer(hbm_budget_bytes=int(0.5 * free), max_batch=32)
    sb = server.run(mixed, realtime=True)
    server.close()
    alone = _serve_requests(kinds, [0.0] * args.requests, geoms, args.maxiter, fwd)
    pb = run_plain(alone)
    same_b = all(torch.equal(a.result, b.result) for a, b in zip(mixed, alone))
    for e in fwd.values():
        e.close()
    out = {"metric": "inversions_per_s", "value": sa["inversions_per_s"], "unit": "inversions/s", "n_gpus": 1,
           "mode": "serve", "higher_is_better": True, "dtype": "f32", "data": "synthetic",
           "config": {"workload": f"{nh} L-BFGS({args.maxiter}) + TV inversions of 70x70, 5 shots, nt={NT}, "
                                  "smoothed starts"},
           "plain_inversions_per_s": pa["inversions_per_s"],
           "speedup_vs_plain": sa["inversions_per_s"] / pa["inversions_per_s"],
           "p50_latency_s": sa["p50_latency_s"], "p99_latency_s": sa["p99_latency_s"],
           "results_identical_served_and_plain": same_a, "served": sa, "plain": pa,
           "stream": {"workload": f"Poisson, {args.requests} requests at {args.rate}/s, mix {SERVE_MIX}",
                      "inversions_per_s": sb["inversions_per_s"], "p50_latency_s": sb["p50_latency_s"],
                      "p99_latency_s": sb["p99_latency_s"], "one_at_a_time_inversions_per_s": pb["inversions_per_s"],
                      "results_identical_alone_and_in_the_mix": same_b, "server": sb}}
    print(json.dumps(out))


HETERO_GRIDS = [(70, 70), (100, 140), (200, 300), (350, 500)]


def run_hetero(args):
    """Config 3: 48 models on grids {70x70, 100x140, 200x300, 350x500}, 5-20 shots, nt in
    {1000, 1500, 2000}, forward + adjoint of all of them in one call."""
    import torch

    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    from seismic_gb300.serving import HeterogeneousBatch, shot_workspace_bytes
    torch.cuda.set_device(0)
    rng = np.random.default_rng(7)
    setups = {}
    jobs = []
    shot_steps = 0
    for i in range(48):
        nz, nx = HETERO_GRIDS[int(rng.integers(0, 4))]
        ns = int(rng.choice([5, 10, 20]))
        nt = int(rng.choice([1000, 1500, 2000]))
        g = setups.setdefault((nz, nx, ns, nt), Geometry.surface(nz, nx, ns, nt))
        v = synthetic.model(rng, ["layered", "faulted"][i % 2], nz, nx)
        jobs.append((g, torch.as_tensor(synthetic.to_vector(v), device="cuda"),
                     torch.as_tensor(rng.normal(0, 1e-3, g.nrecords), device="cuda")))
        shot_steps += ns * nt * 2
    def timed(hb):
        first = hb.run(jobs)
        torch.cuda.synchronize()
        times = []
        for _ in range(max(1, args.steps)):
            t0 = time.perf_counter()
            hb.run(jobs)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        # sweep launches of the call: rounds of chunks x (forward + reverse) in the one-launch
        # form, every engine's own launches otherwise
        infos = [(g.engine.info("last_fwd_launches"), g.engine.info("last_adj_launches")) for g in hb.groups.values()]
        launches = 2 * max(f for f, _ in infos) if hb.one_launch else sum(f + a for f, a in infos)
        return statistics.median(times), first, launches

    # each set-up's engine on its own stream (the default form: cluster sweeps for 70x70,
    # graphs of step launches elsewhere), and beside it one persistent wavefront launch per
    # sweep for all 25 set-ups
    hb1 = HeterogeneousBatch(max_models=48)
    t, out1, sweeps1 = timed(hb1)
    plan1 = {"checkpointed_setups": sum(1 for grp in hb1.groups.values() if grp.checkpoint_every),
             "workspace_gb": round(sum(grp.engine.info("slots") * shot_workspace_bytes(grp.geometry, grp.checkpoint_every)
                                       for grp in hb1.groups.values()) / 1e9, 1)}
    for grp in hb1.groups.values():
        grp.engine.close()
    hb1.groups.clear()
    torch.cuda.empty_cache()
    hb2 = HeterogeneousBatch(max_models=48, one_launch=True)
    t2, out2, sweeps2 = timed(hb2)
    same = all(torch.equal(a[0], b[0]) and torch.equal(a[1], b[1]) for a, b in zip(out1, out2))
    out = {"metric": "shot_steps_per_s", "value": shot_steps / t, "unit": "shot-steps/s", "mode": "hetero",
           "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
           "config": {"workload": "48 models, grids {70x70,100x140,200x300,350x500}, 5-20 shots, nt {1000,1500,2000}",
                      "distinct_setups": len(setups), "form": "each set-up's engine on its own stream",
                      "memory_plan": plan1},
           "s_per_call": t, "models_per_s": 48 / t, "sweep_launches_per_call": sweeps1,
           "one_launch": {"s_per_call": t2, "value": shot_steps / t2, "sweep_launches_per_call": sweeps2,
                          "what": "all set-ups in one persistent wavefront launch per sweep"},
           "results_identical": same}
    print(json.dumps(out))


def run_wave(args):
    """The tiled sweeps as graphs of step launches (sweep_path 1) against one persistent
    wavefront launch per sweep (sweep_path 3): cost + gradient on the uneven batch's grids,
    device time of each sweep (CUDA events), results compared bitwise."""
    import torch

    from seismic_gb300 import synthetic
    from seismic_gb300.engine import Engine
    from seismic_gb300.geometry import Geometry
    torch.cuda.set_device(0)
    cases = [("70x70", 70, 70, 5, 1000, 8, 0), ("100x140", 100, 140, 10, 1000, 4, 0),
             ("200x300", 200, 300, 10, 1500, 2, 0), ("350x500", 350, 500, 10, 2000, 1, 50)]
    out = {"metric": "sweep_ms", "mode": "wave", "unit": "ms per sweep (forward, reverse)", "n_gpus": 1,
           "higher_is_better": False, "dtype": "f32", "data": "synthetic", "cases": {}}
    for name, nz, nx, ns, nt, m, ck in cases:
        g = Geometry.surface(nz, nx, ns, nt)
        rng = np.random.default_rng(5)
        v = torch.as_tensor(np.stack([synthetic.to_vector(synthetic.model(rng, "faulted", nz, nx)) for _ in range(m)]),
                            device="cuda")
        w = torch.as_tensor(rng.normal(0, 1e-3, (m, g.nrecords)), device="cuda")
        eng = Engine(g, max_models=m)
        eng.set_option("checkpoint_every", ck)
        res, row = {}, {"models": m, "shots": ns, "nt": nt, "checkpoint_every": ck}
        for path in (1, 3):
            eng.set_option("sweep_path", path)
            for _ in range(1 + max(1, args.steps)):
                r = eng.vel_to_seis(v, None, w)
            st = eng.stats()
            eng.check()
            res[path] = [a.cpu() for a in r if a is not None]
            row["step_launches" if path == 1 else "wavefront"] = [round(st["fwd_ms"], 2), round(st["adj_ms"], 2)]
        row["bitwise_equal"] = all(torch.equal(a, b) for a, b in zip(res[1], res[3]))
        out["cases"][name] = row
        eng.close()
    print(json.dumps(out))


def run_gn(args):
    """Config 4 (scaled in iterations): Gauss-Newton-CG with 20 CG matvecs per iteration on
    --gn-models 70x70 (5 shots, nt 1000) and 200x300 (10 shots, nt 1500) models each, from
    2 km Gaussian-smoothed starts, all models of a grid in lockstep (fused gn_matvec calls);
    beside it one 70x70 model through the single-model two-call form."""
    import torch

    from seismic_gb300 import inversion, priors, synthetic
    from seismic_gb300.engine import Engine
    from seismic_gb300.geometry import Geometry
    torch.cuda.set_device(0)
    rng = np.random.default_rng(17)
    m = args.gn_models
    out = {"metric": "gn_model_iterations_per_s", "unit": "model GN iterations/s", "mode": "gn", "n_gpus": 1,
           "higher_is_better": True, "dtype": "f32", "data": "synthetic",
           "config": {"workload": f"{m} x 70x70 (5 shots, nt 1000) + {m} x 200x300 (10 shots, nt 1500), "
                                  f"{args.gn_iters} GN iterations x 20 CG matvecs, 2 km smoothed starts, RowTV prior"},
           "grids": {}}
    total_t = 0.0
    for name, g in (("70x70", Geometry.reference(nt=1000)), ("200x300", Geometry.surface(200, 300, 10, 1500))):
        trues = [synthetic.model(rng, ["layered", "faulted", "curved"][i % 3], g.nz, g.nx) for i in range(m)]
        eng = Engine(g, max_models=max(m, 32))
        tv = torch.as_tensor(np.stack([synthetic.to_vector(v) for v in trues]), device="cuda")
        targets = eng.vel_to_seis(tv)[0]
        sig = 2000.0 / g.dx
        starts = torch.as_tensor(np.stack([synthetic.to_vector(synthetic.smoothed(v, sig), v.min()) for v in trues]),
                                 device="cuda")
        pr = priors.RowTotalVariation(g.nz, g.nx, device="cuda").prep()
        pr.lam = 1e-8
        # warm-up with the whole batch: the engine captures its sweep graphs for this chunk once
        inversion.seis_to_vel_gn_cg_batched(targets, starts, pr, eng, n_outer=1, n_cg=1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, hist = inversion.seis_to_vel_gn_cg_batched(targets, starts, pr, eng, n_outer=args.gn_iters, n_cg=20)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        total_t += t
        entry = {"models": m, "s": t, "model_iterations_per_s": m * args.gn_iters / t,
                 "cost_ratio_mean": float(np.mean(hist[-1] / hist[0]))}
        if name == "70x70":
            t0 = time.perf_counter()
            inversion.seis_to_vel_gn_cg(targets[0].reshape(-1, 1), starts[0].reshape(-1, 1), pr, eng,
                                        n_outer=1, n_cg=20)
            torch.cuda.synchronize()
            entry["plain_s_per_iteration"] = time.perf_counter() - t0
            entry["speedup_vs_plain"] = entry["model_iterations_per_s"] * entry["plain_s_per_iteration"]
        out["grids"][name] = entry
        eng.close()
    out["value"] = 2 * m * args.gn_iters / total_t
    print(json.dumps(out))


def _rank_entry(local, world, port):
    os.environ.update(RANK=str(local), LOCAL_RANK=str(local), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    main()


def spawn_ranks(n):
    """``--gpus N`` without a launcher: start N ranks (one per GPU) on this node, as
    torchrun would, each running this benchmark with RANK / LOCAL_RANK / WORLD_SIZE set."""
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    mp.spawn(_rank_entry, args=(n, port), nprocs=n, join=True)


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        spawn_ranks(args.gpus)
        return
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.mode == "serve":
        run_serve(args)
    elif args.mode == "hetero":
        run_hetero(args)
    elif args.mode == "wave":
        run_wave(args)
    elif args.mode == "gn":
        run_gn(args)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
