"""GPU: the persistent wavefront sweeps (sweep_path 3: one launch per sweep, items of
(stage, shot slot, tile) waiting on their neighbour tiles) against the graph of tiled
step launches (sweep_path 1): records, tangent records, gradients and misfits bitwise
equal, whole history and checkpointed, fused and single steps, one and several groups
and chunks; and the multi-geometry call that sweeps several engines' batches in one
forward and one reverse launch."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as _t
    assert _t.cuda.is_available(), "GPU tests need CUDA"
    return _t


def _model(seed, nz, nx, family="faulted"):
    from seismic_gb300 import synthetic
    return synthetic.to_vector(synthetic.model(np.random.default_rng(seed), family, nz, nx))


def _run(torch, eng, vecs, vd=None, w=None, resid=False, misfit=False):
    t = lambda a: None if a is None else torch.as_tensor(np.asarray(a, np.float64), device="cuda")
    out = eng.vel_to_seis(t(vecs), t(vd), t(w), adjoint_on_residual=resid, want_misfit=misfit)
    torch.cuda.synchronize()
    eng.check()
    return [None if a is None else a.cpu().numpy() for a in out]


def _same(a, b):
    return all((x is None and y is None) or np.array_equal(x, y) for x, y in zip(a, b))


GEOMS = {
    "70x70": dict(nz=70, nx=70, nbc=120, nt=301, source_x_cells=(0, 17, 34, 52, 69)),
    "100x140": dict(nz=100, nx=140, nbc=120, nt=201, source_x_cells=(0, 47, 139),
                    receiver_x_cells=tuple(range(0, 140, 3))),
    "ragged_odd": dict(nz=33, nx=65, nbc=20, nt=250, source_x_cells=(64,), source_z_cell=2,
                       receiver_x_cells=tuple(range(0, 65, 4))),
    "below_one_tile": dict(nz=5, nx=7, nbc=10, nt=160, source_x_cells=(0, 6), source_z_cell=0,
                           receiver_x_cells=(0, 3, 6)),
}


@pytest.mark.parametrize("name", list(GEOMS))
def test_wave_sweeps_match_step_launches(torch, name):
    from seismic_gb300.engine import Engine
    from seismic_gb300.geometry import Geometry
    g = Geometry(**GEOMS[name])
    m = 3
    vecs = np.stack([_model(60 + i, g.nz, g.nx, ("faulted", "layered", "curved")[i]) for i in range(m)])
    rng = np.random.default_rng(61)
    vd = rng.normal(0, 1.0, (m, g.nv))
    w = rng.normal(0, 1e-2, (m, g.nrecords))
    for chunk in (0, 2):            # one chunk, and chunks of 2 shot slots (progress reused)
        eng = Engine(g, max_models=m, max_shots_per_chunk=chunk)
        eng.set_option("sweep_path", 1)
        ref_fwd = _run(torch, eng, vecs)
        ref_tan = _run(torch, eng, vecs, vd)
        ref_adj = _run(torch, eng, vecs, None, w, resid=True, misfit=True)
        eng.set_option("checkpoint_every", 25)
        ref_ck = _run(torch, eng, vecs, None, w, resid=True, misfit=True)
        eng.set_option("checkpoint_every", 0)
        eng.set_option("sweep_path", 3)
        for gs in (0, 1):           # automatic group size, and one slot per group
            eng.set_option("wave_group_slots", gs)
            assert _same(_run(torch, eng, vecs), ref_fwd)
            assert eng.info("last_fwd_path") == 3
            chunks = -(-m * g.nshots // eng.info("slots"))
            assert eng.info("last_fwd_launches") == chunks
            assert _same(_run(torch, eng, vecs, vd), ref_tan)
            assert _same(_run(torch, eng, vecs, None, w, resid=True, misfit=True), ref_adj)
            assert eng.info("last_adj_path") == 3 and eng.info("last_adj_launches") == chunks
            eng.set_option("checkpoint_every", 25)
            assert _same(_run(torch, eng, vecs, None, w, resid=True, misfit=True), ref_ck)
            assert eng.info("last_adj_launches") == chunks
            eng.set_option("checkpoint_every", 0)
        assert eng.info("err_word") == 0
        eng.close()


def test_wave_gn_matvec_matches_step_launches(torch):
    from seismic_gb300.engine import Engine
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=301)
    vecs = np.stack([_model(70, 70, 70), _model(71, 70, 70, "layered")])
    vd = np.random.default_rng(72).normal(0, 1.0, (2, g.nv))
    eng = Engine(g, max_models=2)
    t = lambda a: torch.as_tensor(a, device="cuda")
    eng.set_option("sweep_path", 1)
    ref = [a.cpu().numpy() for a in eng.gn_matvec(t(vecs), t(vd))]
    eng.set_option("sweep_path", 3)
    got = [a.cpu().numpy() for a in eng.gn_matvec(t(vecs), t(vd))]
    torch.cuda.synchronize()
    eng.check()
    assert all(np.array_equal(a, b) for a, b in zip(ref, got))


def test_wave_large_grid_matches_step_launches(torch):
    """200x300 (440x540 padded, 126 tiles per shot), 2 shots, nt 200."""
    from seismic_gb300.engine import Engine
    from seismic_gb300.geometry import Geometry
    g = Geometry.surface(200, 300, 2, 200)
    vec = _model(80, 200, 300)
    w = np.random.default_rng(81).normal(0, 1e-2, g.nrecords)
    eng = Engine(g, max_models=1)
    eng.set_option("sweep_path", 1)
    ref = _run(torch, eng, vec, None, w)
    eng.set_option("sweep_path", 3)
    got = _run(torch, eng, vec, None, w)
    assert _same(got, ref)
    assert rel_l2(got[2], ref[2]) == 0.0


def _multi_case():
    from seismic_gb300.geometry import Geometry
    return [
        (Geometry(**GEOMS["70x70"]), 3, 0, 0),
        (Geometry(**GEOMS["ragged_odd"]), 2, 0, 0),
        (Geometry(**GEOMS["100x140"]), 2, 25, 0),          # checkpointed adjoint
        (Geometry.surface(40, 60, 4, 220, nbc=30), 3, 0, 5),  # 12 shots in chunks of 5: three rounds
    ]


@pytest.mark.parametrize("adjoint", [True, False])
def test_multi_engine_call_matches_each_engine_alone(torch, adjoint):
    """seis_vel_to_seis_multi: four geometries (one checkpointed, one in three chunk
    rounds) in one forward and one reverse launch per round give bitwise each engine's
    own records, gradients and misfits."""
    from seismic_gb300.engine import Engine, vel_to_seis_multi
    engines, vecs, tgts, alone = [], [], [], []
    for k, (g, m, ck, chunk) in enumerate(_multi_case()):
        eng = Engine(g, max_models=m, max_shots_per_chunk=chunk)
        if ck:
            eng.set_option("checkpoint_every", ck)
        rng = np.random.default_rng(90 + k)
        v = np.stack([_model(91 + 3 * k + i, g.nz, g.nx, ("faulted", "layered", "curved")[i]) for i in range(m)])
        tg = rng.normal(0, 1e-3, (m, g.nrecords))
        eng.set_option("sweep_path", 1)
        alone.append(_run(torch, eng, v, None, tg if adjoint else None, resid=adjoint, misfit=adjoint))
        engines.append(eng)
        vecs.append(torch.as_tensor(v, device="cuda"))
        tgts.append(torch.as_tensor(tg, device="cuda"))
    outs = vel_to_seis_multi(engines, vecs, tgts if adjoint else None, adjoint_on_residual=adjoint,
                             want_misfit=adjoint)
    torch.cuda.synchronize()
    for eng, (res, ra, mf), ref in zip(engines, outs, alone):
        eng.check()
        assert np.array_equal(res.cpu().numpy(), ref[0])
        if adjoint:
            assert np.array_equal(ra.cpu().numpy(), ref[2]) and np.array_equal(mf.cpu().numpy(), ref[3])
        assert eng.info("last_fwd_path") == 3
    rounds = [-(-m * g.nshots // e.info("slots")) for (g, m, _, _), e in zip(_multi_case(), engines)]
    assert rounds == [1, 1, 1, 3]
    assert [e.info("last_fwd_launches") for e in engines] == rounds
    # the same arrays twice, or one engine twice, are refused
    with pytest.raises(Exception):
        vel_to_seis_multi([engines[0], engines[0]], [vecs[0], vecs[0]])
    for e in engines:
        e.close()


def test_heterogeneous_batch_one_launch_matches_per_engine_calls(torch):
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    from seismic_gb300.serving import HeterogeneousBatch
    rng = np.random.default_rng(95)
    jobs = []
    for i, (nz, nx, ns, nt) in enumerate([(70, 70, 5, 300), (40, 60, 3, 250), (70, 70, 5, 300), (60, 90, 4, 200)]):
        g = Geometry.surface(nz, nx, ns, nt)
        v = synthetic.to_vector(synthetic.model(rng, "faulted", nz, nx))
        jobs.append((g, torch.as_tensor(v, device="cuda"), torch.as_tensor(rng.normal(0, 1e-3, g.nrecords),
                                                                             device="cuda")))
    one = HeterogeneousBatch(max_models=4, one_launch=True).run(jobs)
    per = HeterogeneousBatch(max_models=4, one_launch=False).run(jobs)
    for (m1, g1), (m2, g2) in zip(one, per):
        assert np.array_equal(m1.cpu().numpy(), m2.cpu().numpy())
        assert np.array_equal(g1.cpu().numpy(), g2.cpu().numpy())
