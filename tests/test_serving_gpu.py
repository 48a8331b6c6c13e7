"""GPU: continuous batching of whole inversions and heterogeneous batches."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as _t
    assert _t.cuda.is_available()
    return _t


def _requests(torch, n, maxiter=4):
    from seismic_gb300 import priors, synthetic
    from seismic_gb300.engine import Engine
    from seismic_gb300.geometry import Geometry
    from seismic_gb300.serving import InversionRequest
    geoms = [Geometry(nz=30, nx=40, nbc=30, nt=300, source_x_cells=(0, 20, 39)),
             Geometry(nz=24, nx=50, nbc=30, nt=250, source_x_cells=(0, 25, 49))]
    engines = [Engine(g, max_models=1) for g in geoms]
    rng = np.random.default_rng(21)
    reqs = []
    for i in range(n):
        k = i % 2
        g = geoms[k]
        vt = synthetic.model(rng, ["layered", "curved"][k], g.nz, g.nx)
        v0 = synthetic.smoothed(vt, 2.0)
        tgt = engines[k].vel_to_seis(torch.as_tensor(synthetic.to_vector(vt), device="cuda"))[0][0]
        pr = priors.TotalVariation(g.nz, g.nx, device="cuda")
        pr.lam = 1e-6
        pr.prep()
        reqs.append(InversionRequest(rid=i, geometry=g, target=tgt,
                                     start=torch.as_tensor(synthetic.to_vector(v0, vt.min()), device="cuda"),
                                     prior=pr, maxiter=maxiter, arrival=0.05 * i))
    return reqs


@pytest.mark.parametrize("lanes,share", [(1, None), (2, None), (2, True)])
def test_results_are_the_same_alone_and_in_the_mix(torch, lanes, share):
    """Requests served together (two grid sizes, memory-limited admission, one or two
    lanes per grid, the lanes with their own engines or sharing one) give bitwise the
    models they give one at a time."""
    from seismic_gb300.serving import InversionServer, run_plain
    mixed = _requests(torch, 6)
    alone = _requests(torch, 6)
    server = InversionServer(hbm_budget_bytes=0, lanes=lanes, share_lane_engines=share)
    server.budget = 3 * max(server.footprint(r) for r in mixed)     # at most 3 requests resident
    # all released at once: three are admitted, the others join as memory frees up
    stats = server.run(mixed, realtime=False)
    run_plain(alone)
    assert stats["max_active"] == 3
    if lanes == 1:
        assert stats["engine_calls"] < stats["evaluations"]         # requests shared calls
    admitted = sorted(r.admitted for r in mixed)
    assert admitted[3] > admitted[0]                                 # the fourth waited for a slot
    for a, b in zip(mixed, alone):
        assert a.result is not None and torch.equal(a.result, b.result), a.rid
        assert a.evaluations == b.evaluations
    assert all(np.isfinite(r.latency) and r.latency > 0 for r in mixed)


def test_heterogeneous_batch_matches_single_engines(torch):
    from seismic_gb300 import synthetic
    from seismic_gb300.engine import Engine
    from seismic_gb300.geometry import Geometry
    from seismic_gb300.serving import HeterogeneousBatch
    geoms = [Geometry(nz=20, nx=30, nbc=20, nt=200, source_x_cells=(0, 29)),
             Geometry(nz=28, nx=22, nbc=25, nt=260, source_x_cells=(5, 15)),
             Geometry.reference(nt=300)]
    rng = np.random.default_rng(4)
    jobs = []
    for i in range(7):
        g = geoms[i % 3]
        v = torch.as_tensor(synthetic.to_vector(synthetic.model(rng, "faulted", g.nz, g.nx)), device="cuda")
        t = torch.as_tensor(rng.normal(0, 1e-2, g.nrecords), device="cuda")
        jobs.append((g, v, t))
    hb = HeterogeneousBatch(max_models=2)
    out = hb.run(jobs)
    assert not any(grp.checkpoint_every for grp in hb.groups.values())     # whole histories fit
    # memory for no whole history: every set-up checkpointed, in chunks that fill the GPU
    tight = HeterogeneousBatch(max_models=2, memory_fraction=1e-9)
    out_ck = tight.run(jobs)
    assert all(grp.checkpoint_every == 50 for grp in tight.groups.values())
    for (g, v, t), (mf, gr), (mf2, gr2) in zip(jobs, out, out_ck):
        _, _, g1, m1 = Engine(g, max_models=1).vel_to_seis(v, None, t, adjoint_on_residual=True, want_misfit=True)
        assert torch.equal(gr, g1[0]) and torch.equal(mf, m1[0])
        assert torch.equal(gr2, g1[0]) and torch.equal(mf2, m1[0])


def test_fused_tv_prior_kernel(torch):
    """The library's TV prior kernel equals the restated prior and does not depend on
    how many models share the call."""
    from seismic_gb300 import priors
    pr = priors.TotalVariation(23, 31, device="cuda")
    pr.lam = 7.0
    pr.prep()
    X = torch.as_tensor(np.random.default_rng(1).normal(2000, 50, (5, pr.N)), device="cuda")
    c, g = pr.batched_cost_and_gradient(X)
    for i in range(5):
        ci, gi = pr.compute_cost_and_gradient(X[i][:, None], compute_gradient=True)
        assert abs(float(c[i]) / float(ci) - 1) < 1e-12
        assert float((g[i] - gi[:, 0]).abs().max()) <= 1e-12 * float(gi.abs().max())
        c1, g1 = pr.batched_cost_and_gradient(X[i:i + 1])
        assert torch.equal(c1[0], c[i]) and torch.equal(g1[0], g[i])


def test_served_step_reports_a_timed_out_wait(torch):
    """A served evaluation whose cluster adjoint gives up a bounded wait (a history copy
    withheld by the engine's test hook) raises SeisError in the serving loop, which reads
    the engine's error word where it already waits for each call; the engine recovers."""
    from seismic_gb300 import priors, synthetic
    from seismic_gb300._lib import SeisError
    from seismic_gb300.geometry import Geometry
    from seismic_gb300.serving import InversionRequest, InversionServer
    g = Geometry.reference(nt=200)
    rng = np.random.default_rng(5)

    def request(i):
        vt = synthetic.model(rng, "layered", g.nz, g.nx)
        pr = priors.RowTotalVariation(g.nz, g.nx, device="cuda").prep()
        tgt = torch.as_tensor(rng.normal(0, 1e-3, g.nrecords), device="cuda")
        return InversionRequest(rid=i, geometry=g, target=tgt, prior=pr, maxiter=2,
                                start=torch.as_tensor(synthetic.to_vector(synthetic.smoothed(vt, 2.0), vt.min()),
                                                      device="cuda"))

    free, _ = torch.cuda.mem_get_info()
    server = InversionServer(hbm_budget_bytes=int(0.3 * free), max_geometries=1, lanes=1)
    server.run([request(0)], realtime=False)                     # creates the engine
    (grp,) = server.groups.values()
    assert grp.engine.info("cluster_adj") > 0
    grp.engine.set_option("test_skip_history_copy", 0)
    with pytest.raises(SeisError) as ei:
        server.run([request(1)], realtime=False)
    assert ei.value.status == -5
    grp.engine.set_option("test_skip_history_copy", -1)
    server.active.clear()
    server.used = 0
    stats = server.run([request(2)], realtime=False)
    assert stats["evaluations"] >= 1
    grp.engine.check()
    server.close()
