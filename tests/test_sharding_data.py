"""CPU: shot-sharded evaluation over gloo ranks, failure of a rank, and the data formats."""
import datetime
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest
import torch


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _problem(nshots=5):
    from oracle import oracle
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    g = Geometry(nz=16, nx=22, nbc=12, nt=180, source_x_cells=(0, 5, 11, 16, 21)[:nshots])
    rng = np.random.default_rng(3)
    vec = synthetic.to_vector(synthetic.model(rng, "curved", 16, 22))[:, None]
    tgt = oracle.vel_to_seis(g, synthetic.to_vector(synthetic.model(rng, "layered", 16, 22))[:, None])[0]
    return g, vec, tgt


def _rank_main(rank, world, port, out, fail_rank):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=8))
    from oracle import oracle
    from seismic_gb300.sharding import record_slice, reduce_evaluation, shard_shots, shot_subset
    g, vec, tgt = _problem()
    shots = shard_shots(g.nshots, world, rank)
    local = shot_subset(g, shots)
    t = tgt[record_slice(g, shots)]
    res, _, grad = oracle.vel_to_seis(local, vec, None, t, adjoint_on_residual=True)
    misfit = torch.tensor(float(np.sum((res - t) ** 2)), dtype=torch.float64)
    gr = torch.as_tensor(grad[:, 0])
    if rank == fail_rank:
        os._exit(3)                      # a rank dies between steps, before the exchange
    try:
        reduce_evaluation(misfit, gr)
        out.put((rank, "ok", float(misfit), gr.numpy()))
    except Exception as e:              # the survivors learn of it from the group timeout
        out.put((rank, "error", type(e).__name__, None))


def _oracle_sweep(local, vec, t):
    """Stands in for the engine's sweep of a rank's shots: FP64 misfit and gradient."""
    from oracle import oracle
    t = np.asarray(t)
    res, _, grad = oracle.vel_to_seis(local, np.asarray(vec)[:, None], None, t[:, None], adjoint_on_residual=True)
    return torch.tensor(float(np.sum((res[:, 0] - t) ** 2)), dtype=torch.float64), torch.as_tensor(grad[:, 0])


def _evaluator_main(rank, world, port, out, nshots):
    """A rank of ShardedEvaluator.evaluate: its shots swept by the oracle, then the
    evaluator's own all-reduce."""
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=30))
    from seismic_gb300.sharding import ShardedEvaluator
    g, vec, tgt = _problem(nshots)
    ev = ShardedEvaluator(g, sweep=_oracle_sweep)
    mf, gr = ev.evaluate(torch.as_tensor(vec[:, 0]), torch.as_tensor(tgt[:, 0]))
    out.put((rank, len(ev.shots), float(mf), gr.numpy()))
    dist.destroy_process_group()


def _run(world, fail_rank=-1, target=None, extra=()):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    target = target or _rank_main
    args = extra if target is not _rank_main else (fail_rank,)
    ps = [ctx.Process(target=target, args=(r, world, port, q, *args)) for r in range(world)]
    for p in ps:
        p.start()
    res = []
    for _ in range(world - (1 if fail_rank >= 0 else 0)):
        res.append(q.get(timeout=120))
    for p in ps:
        p.join(timeout=60)
    return sorted(res, key=lambda r: r[0])


def test_shot_sharded_gradient_over_two_gloo_ranks():
    """Two ranks sweep shots {0,1,2} and {3,4}; one all-reduce gives the full evaluation."""
    from oracle import oracle
    g, vec, tgt = _problem()
    res, _, grad = oracle.vel_to_seis(g, vec, None, tgt, adjoint_on_residual=True)
    full_mf = float(np.sum((res - tgt) ** 2))
    out = _run(2)
    for rank, status, mf, gr in out:
        assert status == "ok"
        assert abs(mf / full_mf - 1) < 1e-12
        assert np.linalg.norm(gr - grad[:, 0]) / np.linalg.norm(grad) < 1e-12


@pytest.mark.parametrize("world,nshots", [(2, 5), (3, 2)])
def test_sharded_evaluator_over_gloo_ranks(world, nshots):
    """ShardedEvaluator.evaluate end to end on gloo ranks, the oracle standing in for the
    engine's sweep of each rank's shots: every rank gets the full misfit and gradient.
    With more ranks than shots (3 ranks, 2 shots) the rank without shots creates no
    engine, adds zeros and still joins the one all-reduce."""
    from oracle import oracle
    g, vec, tgt = _problem(nshots)
    res, _, grad = oracle.vel_to_seis(g, vec, None, tgt, adjoint_on_residual=True)
    full_mf = float(np.sum((res - tgt) ** 2))
    out = _run(world, target=_evaluator_main, extra=(nshots,))
    assert sum(o[1] for o in out) == nshots and (world <= nshots or min(o[1] for o in out) == 0)
    for rank, nsh, mf, gr in out:
        assert abs(mf / full_mf - 1) < 1e-12
        assert np.linalg.norm(gr - grad[:, 0]) / np.linalg.norm(grad) < 1e-12


def test_dead_rank_is_reported_not_hung():
    """A rank that exits before the exchange: the other rank's all-reduce fails with an
    error after the group timeout instead of waiting forever."""
    out = _run(2, fail_rank=1)
    assert out[0][0] == 0 and out[0][1] == "error"


def test_shard_shots_partition():
    from seismic_gb300.sharding import shard_shots
    for n in (1, 5, 7, 20):
        for w in (1, 2, 3, 4):
            parts = [list(shard_shots(n, w, r)) for r in range(w)]
            assert sum(parts, []) == list(range(n))
            assert max(map(len, parts)) - min(map(len, parts)) <= 1


def test_data_formats(tmp_path):
    """Seismogram / Velocity: .npy stacks, the 999-row truncation and the vector layouts
    (core/kaggle_support.py:192-253)."""
    from seismic_gb300.data import Seismogram, Velocity
    rng = np.random.default_rng(0)
    seis = rng.normal(0, 1, (3, 5, 1000, 70)).astype(np.float32)
    vel = rng.uniform(1500, 4500, (3, 1, 70, 70)).astype(np.float32)
    np.save(tmp_path / "seis.npy", seis)
    np.save(tmp_path / "vel.npy", vel)
    s = Seismogram(str(tmp_path / "seis.npy"), ind=1).load_to_memory(device="cpu")
    assert tuple(s.data.shape) == (5, 999, 70) and np.array_equal(s.data.numpy(), seis[1, :, :999].astype(np.float64))
    s2 = Seismogram(str(tmp_path / "seis.npy"), ind=1).load_to_memory(load_last_row=True, device="cpu")
    assert tuple(s2.data.shape) == (5, 1000, 70)
    v = s.to_vector()
    assert tuple(v.shape) == (349650, 1)
    assert torch.equal(Seismogram().from_vector(v).data, s.data)
    m = Velocity(str(tmp_path / "vel.npy"), ind=2).load_to_memory(device="cpu")
    assert float(m.min_vel) == float(vel[2, 0].min())
    mv = m.to_vector()
    assert tuple(mv.shape) == (4901, 1) and float(mv[-1, 0]) == float(m.min_vel)
    m2 = Velocity().from_vector(mv)
    assert torch.equal(m2.data, m.data) and float(m2.min_vel) == float(m.min_vel)
