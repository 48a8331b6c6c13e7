"""GPU parity: the CUDA engine, called through the C ABI, against the FP64
oracle and against the reference's golden vectors.

Tolerances (relative L2, FP32 sweeps against FP64): records <= 1e-5,
tangent records and gradients <= 1e-4.
"""
import numpy as np
import pytest

from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu

REC_TOL = 1e-5
GRAD_TOL = 1e-4
TAN_TOL = 1e-4


@pytest.fixture(scope="module")
def torch():
    import torch as _t
    assert _t.cuda.is_available(), "GPU tests need CUDA"
    return _t


def _engine(geom, nmodels=1, chunk=0):
    from seismic_gb300.engine import Engine
    return Engine(geom, max_models=nmodels, max_shots_per_chunk=chunk)


def _run(torch, eng, vecs, vd=None, w=None, resid=False, misfit=False):
    dev = "cuda"
    t = lambda a: None if a is None else torch.as_tensor(np.asarray(a, np.float64), device=dev)
    res, rd, ra, mf = eng.vel_to_seis(t(vecs), t(vd), t(w), adjoint_on_residual=resid, want_misfit=misfit)
    torch.cuda.synchronize()
    c = lambda a: None if a is None else a.cpu().numpy()
    return c(res), c(rd), c(ra), c(mf)


def _model(seed, nz, nx, family="faulted"):
    from seismic_gb300 import synthetic
    return synthetic.to_vector(synthetic.model(np.random.default_rng(seed), family, nz, nx))


@pytest.mark.parametrize("case", ["ref70_layered", "ref70_faulted_residual"])
def test_reference_golden(torch, parity_report, case):
    """Reference geometry (70x70, nt=999, 5 shots): records, tangent and gradient
    against the reference's own FP64 output."""
    from seismic_gb300.geometry import Geometry
    gd = load_golden(case)
    g = Geometry.reference()
    vec = gd["vec"]
    w = np.random.default_rng(int(gd["adjoint_seed"])).normal(0.0, float(gd["adjoint_sigma"]), g.nrecords)
    vd = None
    if "tangent_seed" in gd:
        vd = np.random.default_rng(int(gd["tangent_seed"])).normal(0.0, 1.0, g.nv)
    res, rd, ra, _ = _run(torch, _engine(g), vec, vd, w, resid=bool(gd["adjoint_on_residual"]))
    s = int(gd["row_stride"])
    errs = dict(records=rel_l2(res.reshape(5, 999, 70)[:, ::s], gd["rec_rows"]), gradient=rel_l2(ra[0], gd["grad"]))
    if vd is not None:
        errs["tangent"] = rel_l2(rd.reshape(5, 999, 70)[:, ::s], gd["drec_rows"])
    # every record row (the stored rows are every 10th time step, all even; the two-step
    # kernels write the odd ones separately): each row's L2 norm and sum against the
    # reference's per-row moments, relative to the shot's largest row norm
    for out, key in ((res, "rec"), (rd, "drec")):
        if out is not None:
            r = out.reshape(5, 999, 70)
            rn = np.sqrt(gd[f"{key}_row_sumsq"])
            top = rn.max(axis=1, keepdims=True)
            errs[f"{key}_every_row"] = float(max(np.max(np.abs(np.sqrt((r ** 2).sum(axis=2)) - rn) / top),
                                                 np.max(np.abs(r.sum(axis=2) - gd[f"{key}_row_sum"]) / (np.sqrt(70) * top))))
    parity_report(f"{case} (vs the reference's own output)", **errs)
    assert errs["records"] < REC_TOL
    assert abs((res ** 2).sum() / gd["rec_sumsq"] - 1) < 2 * REC_TOL
    assert errs["gradient"] < GRAD_TOL
    # a row's error is at most the whole record's: at the measured relative errors (about
    # 6e-7 records, 8e-6 tangent) and 4995 rows, at most about 4e-5 and 6e-4 of the largest
    # row norm (measured per row: 2e-7 and 3e-6); a wrong row the stored tenth leaves out
    # exceeds these bounds
    assert errs["rec_every_row"] < 1e-4
    if vd is not None:
        assert errs["tangent"] < TAN_TOL
        assert errs["drec_every_row"] < 1e-3


def test_reference_geometry_nt1000_vs_oracle(torch, oracle, parity_report):
    """Full records, tangent and gradient at 70x70 / nt=1000 (the benchmark's model size)."""
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=1000)
    vec = _model(31, 70, 70, "curved")
    rng = np.random.default_rng(32)
    vd = rng.normal(0, 10, g.nv)
    vt = vec * (1 + 0.03 * np.sin(np.arange(g.nv) / 50.0))
    t_rec = oracle.vel_to_seis(g, vt[:, None])[0][:, 0]
    o_res, o_rd, o_ra = oracle.vel_to_seis(g, vec[:, None], vd[:, None], t_rec[:, None], adjoint_on_residual=True)
    res, rd, ra, mf = _run(torch, _engine(g), vec, vd, t_rec, resid=True, misfit=True)
    parity_report("70x70 nt=1000 shots=5", records=rel_l2(res[0], o_res), tangent=rel_l2(rd[0], o_rd),
                  gradient=rel_l2(ra[0], o_ra), misfit=abs(mf[0] / np.sum((o_res[:, 0] - t_rec) ** 2) - 1))
    assert rel_l2(res[0], o_res) < REC_TOL
    assert rel_l2(rd[0], o_rd) < TAN_TOL
    assert rel_l2(ra[0], o_ra) < GRAD_TOL
    assert abs(mf[0] / np.sum((o_res[:, 0] - t_rec) ** 2) - 1) < 1e-4


SMALL = [
    # nz, nx, nbc, nt, source x cells, source z cell, receiver x cells
    (24, 30, 16, 300, (0, 11, 29), 1, None),
    (5, 7, 10, 160, (0, 6), 0, (0, 3, 6)),                # padded grid narrower than one tile
    (33, 65, 20, 250, (64,), 2, tuple(range(0, 65, 4))),   # ragged tiles, source at the right edge
    (17, 9, 30, 200, (4,), 16, (0, 8)),                    # source at the bottom row of the model
]


@pytest.mark.parametrize("spec", SMALL)
def test_small_geometries_vs_oracle(torch, oracle, spec):
    from seismic_gb300.geometry import Geometry
    nz, nx, nbc, nt, sx, sz, rx = spec
    g = Geometry(nz=nz, nx=nx, nbc=nbc, nt=nt, source_x_cells=sx, source_z_cell=sz, receiver_x_cells=rx)
    vec = _model(40 + nz, nz, nx)
    rng = np.random.default_rng(nz)
    vd = rng.normal(0, 20, g.nv)
    w = rng.normal(0, 1e-2, g.nrecords)
    o = oracle.vel_to_seis(g, vec[:, None], vd[:, None], w[:, None], adjoint_on_residual=False)
    res, rd, ra, _ = _run(torch, _engine(g), vec, vd, w)
    assert rel_l2(res[0], o[0]) < REC_TOL
    assert rel_l2(rd[0], o[1]) < TAN_TOL
    assert rel_l2(ra[0], o[2]) < GRAD_TOL


def test_batch_and_chunking_are_invariant(torch):
    """Several models in one call give bitwise the same outputs as one at a time,
    whatever the number of concurrently swept shots."""
    from seismic_gb300.geometry import Geometry
    g = Geometry(nz=20, nx=26, nbc=10, nt=200, source_x_cells=(0, 9, 25))
    vecs = np.stack([_model(s, 20, 26, f) for s, f in [(1, "layered"), (2, "faulted"), (3, "curved")]])
    w = np.random.default_rng(9).normal(0, 1e-2, (3, g.nrecords))
    full = _run(torch, _engine(g, 3), vecs, None, w, resid=True)
    for chunk in (1, 2, 4):
        part = _run(torch, _engine(g, 3, chunk), vecs, None, w, resid=True)
        assert np.array_equal(full[0], part[0]) and np.array_equal(full[2], part[2])
    for m in range(3):
        one = _run(torch, _engine(g, 1), vecs[m], None, w[m], resid=True)
        assert np.array_equal(full[0][m], one[0][0]) and np.array_equal(full[2][m], one[2][0])


def test_adjoint_dot_product_fp32(torch):
    """<J d, w> = <d, J^T w> for the FP32 tangent and adjoint sweeps."""
    from seismic_gb300.geometry import Geometry
    g = Geometry(nz=30, nx=40, nbc=20, nt=400, source_x_cells=(5, 30))
    vec = _model(5, 30, 40, "curved")
    rng = np.random.default_rng(1)
    d = rng.normal(0, 10, g.nv)
    w = rng.normal(0, 1, g.nrecords)
    _, rd, ra, _ = _run(torch, _engine(g), vec, d, w)
    lhs = float(np.dot(rd[0], w))
    rhs = float(np.dot(ra[0], d))
    assert abs(lhs - rhs) / abs(lhs) < 1e-4


def test_drop_in_vel_to_seis(torch):
    """seismic_gb300.seis_forward2.vel_to_seis: the reference signature, shapes and asserts."""
    from seismic_gb300 import seis_forward2 as sf
    gd = load_golden("ref70_layered")
    vec = torch.as_tensor(gd["vec"][:, None], device="cuda")
    res, rd, ra = sf.vel_to_seis(vec)
    assert res.shape == (349650, 1) and res.dtype == torch.float64 and rd is None and ra is None
    s = int(gd["row_stride"])
    assert rel_l2(res.cpu().numpy().reshape(5, 999, 70)[:, ::s], gd["rec_rows"]) < REC_TOL
    w = torch.zeros((349650, 1), dtype=torch.float64, device="cuda")
    res2, _, ra2 = sf.vel_to_seis(vec, None, w, adjoint_on_residual=True)
    assert ra2.shape == (4901, 1) and torch.equal(res2, res)
    with pytest.raises(AssertionError):
        sf.vel_to_seis(vec[:-1])
    with pytest.raises(AssertionError):
        sf.vel_to_seis(vec.float())


def test_engine_rejects_bad_calls(torch):
    from seismic_gb300._lib import SeisError
    from seismic_gb300.geometry import Geometry
    g = Geometry(nz=10, nx=10, nbc=4, nt=150, source_x_cells=(0,))
    eng = _engine(g, 1)
    vec = torch.full((2, g.nv), 2000.0, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        eng.vel_to_seis(vec)
    with pytest.raises(TypeError):
        eng.vel_to_seis(vec[:1].float())
    with pytest.raises(ValueError):
        eng.vel_to_seis(vec[:1], want_misfit=True)
    assert SeisError(-1, "x").status == -1


def test_cluster_sweeps_match_tiled_sweeps(torch, oracle):
    """The cluster-resident sweeps (shared-memory wavefields, DSMEM halos, TMA-staged
    history) against the tiled per-step sweeps and the oracle at 70x70 / nt=1000."""
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=1000)
    vecs, trues, _ = synthetic.batch(77, 3)
    eng = _engine(g, 3)
    assert eng.info("cluster_fwd") > 0 and eng.info("cluster_adj") > 0
    eng.set_option("sweep_path", 1)
    tgt = _run(torch, eng, trues)[0]
    tiled = _run(torch, eng, vecs, None, tgt, resid=True)
    eng.set_option("sweep_path", 2)
    clus = _run(torch, eng, vecs, None, tgt, resid=True)
    eng.check()
    # every rounding step of the two paths is the same: records and gradients agree bitwise
    assert np.array_equal(clus[0], tiled[0]) and np.array_equal(clus[2], tiled[2])
    o = oracle.vel_to_seis(g, vecs[0][:, None], None, tgt[0][:, None], adjoint_on_residual=True)
    assert rel_l2(clus[0][0], o[0]) < REC_TOL
    assert rel_l2(clus[2][0], o[2]) < GRAD_TOL
    # two slots per cluster in turn (more shots than resident clusters) stay identical
    eng1 = _engine(g, 3, chunk=1)
    eng1.set_option("sweep_path", 2)
    one = _run(torch, eng1, vecs, None, tgt, resid=True)
    assert np.array_equal(one[0], clus[0]) and np.array_equal(one[2], clus[2])


def test_cluster_tangent_matches_tiled_tangent(torch):
    """The cluster-resident forward + tangent sweep gives bitwise the tiled sweep's
    records and tangent records (and, with an adjoint in the same call, gradients)."""
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=800)
    vecs, trues, _ = synthetic.batch(21, 3)
    vd = np.random.default_rng(22).normal(0, 5.0, vecs.shape)
    w = np.random.default_rng(23).normal(0, 1e-2, (3, g.nrecords))
    eng = _engine(g, 3)
    assert eng.info("cluster_tan") > 0
    clus = _run(torch, eng, vecs, vd, w)
    assert eng.info("last_fwd_path") == 2
    eng.set_option("sweep_path", 1)
    tiled = _run(torch, eng, vecs, vd, w)
    assert eng.info("last_fwd_path") == 1
    for a, b in zip(clus[:3], tiled[:3]):
        assert np.array_equal(a, b)


def test_pitch_384_cluster_sweeps_match_tiled_sweeps(torch):
    """100x140 models (340x380 padded, row pitch 384) on the cluster path: the tensor-memory
    forward on 10-CTA clusters and adjoint on 16-CTA clusters give bitwise the tiled
    sweeps' records, misfits and gradients (the tangent stays tiled); full and partial
    chunks, odd nt."""
    from seismic_gb300.geometry import Geometry
    g = Geometry(nz=100, nx=140, nbc=120, nt=201, source_x_cells=(0, 47, 93, 139),
                 receiver_x_cells=tuple(range(0, 140, 2)))
    vecs = np.stack([_model(110 + i, 100, 140, ("faulted", "layered", "curved")[i]) for i in range(3)])
    w = np.random.default_rng(111).normal(0, 1e-2, (3, g.nrecords))
    eng = _engine(g, 3)
    assert eng.info("cluster_fwd10") > 0 and eng.info("cluster_adj") > 0
    eng.set_option("sweep_path", 1)
    ref = _run(torch, eng, vecs, None, w, resid=True, misfit=True)
    ref_fwd = _run(torch, eng, vecs[:2])
    eng.set_option("sweep_path", 0)
    out = _run(torch, eng, vecs, None, w, resid=True, misfit=True)
    assert eng.info("last_fwd_path") == 2 and eng.info("last_adj_path") == 2
    assert eng.info("fwd_cluster") == 10 and eng.info("adj_cluster") == 16
    for a, b in zip(out, ref):
        assert (a is None and b is None) or np.array_equal(a, b)
    assert np.array_equal(_run(torch, eng, vecs[:2])[0], ref_fwd[0])
    for side in (0, 3):
        eng.set_option("adj_side", side)
        eng.set_option("fwd_side", side)
        out = _run(torch, eng, vecs, None, w, resid=True, misfit=True)
        for a, b in zip(out, ref):
            assert (a is None and b is None) or np.array_equal(a, b)


def test_cluster_path_falls_back_where_it_does_not_fit(torch):
    from seismic_gb300._lib import SeisError
    from seismic_gb300.geometry import Geometry
    eng = _engine(Geometry.surface(200, 300, 4, 200))   # 440 x 540 padded: no cluster shape has its pitch
    assert eng.info("cluster_fwd") == 0 and eng.info("cluster_fwd10") == 0 and eng.info("cluster_adj") == 0
    with pytest.raises(SeisError):
        eng.set_option("sweep_path", 2)


def test_sixteen_cta_forward_clusters_match(torch):
    """The 16- and 10-CTA forward instantiations (20- and 32-row bands) give bitwise
    the 8-CTA results."""
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=600)
    vecs, trues, _ = synthetic.batch(5, 2)
    eng = _engine(g, 2)
    assert eng.info("cluster_fwd16") > 0 and eng.info("cluster_fwd10") > 0
    tgt = _run(torch, eng, trues)[0]
    eng.set_option("fwd_cluster", 8)
    a = _run(torch, eng, vecs, None, tgt, resid=True)
    for c in (16, 10):
        eng.set_option("fwd_cluster", c)
        assert eng.info("fwd_cluster") == c
        b = _run(torch, eng, vecs, None, tgt, resid=True)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[2], b[2])


def test_column_pair_sweeps_match_single_columns(torch):
    """Column pairs per thread (even widths) give bitwise the one-column results in
    both sweeps, for both forward cluster sizes."""
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=600)
    vecs, trues, _ = synthetic.batch(6, 2)
    eng = _engine(g, 2)
    assert eng.info("fwd_columns") == 2 and eng.info("adj_columns") == 2
    tgt = _run(torch, eng, trues)[0]
    for c in (8, 10, 16):
        eng.set_option("fwd_cluster", c)
        eng.set_option("columns", 2)
        a = _run(torch, eng, vecs, None, tgt, resid=True)
        eng.set_option("columns", 1)
        assert eng.info("fwd_columns") == 1 and eng.info("adj_columns") == 1
        b = _run(torch, eng, vecs, None, tgt, resid=True)
        eng.check()
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[2], b[2])


def test_neighbour_shuffles_match_shared_loads(torch):
    """The forward sweep whose horizontal neighbours come from the adjacent lanes by warp
    shuffles gives bitwise the records and history (so the gradient) of the one that
    loads them from shared memory."""
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=600)
    vecs, trues, _ = synthetic.batch(8, 2)
    eng = _engine(g, 2)
    eng.set_option("fwd_cluster", 10)
    tgt = _run(torch, eng, trues)[0]
    a = _run(torch, eng, vecs, None, tgt, resid=True)
    assert eng.info("fwd_shuffle") == 0
    eng.set_option("neighbour_shuffle", 1)
    assert eng.info("fwd_shuffle") == 1
    b = _run(torch, eng, vecs, None, tgt, resid=True)
    eng.check()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[2], b[2])


@pytest.mark.parametrize("rows", [8, 11])
def test_tensor_memory_adjoint_matches(torch, rows):
    """The 10-CTA cluster adjoint that keeps alpha, the gradient sums and the carried
    history level in tensor memory (8 rows x 640 threads or 11 rows x 480 threads per
    CTA) gives bitwise the 16-CTA register adjoint's gradients and misfits: full and
    partial chunks, with the side adjoint beside it; a withheld history copy makes its
    bounded wait give up, the status says so, and the next call is correct again."""
    from seismic_gb300._lib import SeisError
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=400)
    vecs, trues, _ = synthetic.batch(91, 4)
    eng = _engine(g, 4)
    tgt = _run(torch, eng, trues)[0]
    eng.set_option("adj_side", 0)
    eng.set_option("adj_cluster", 16)
    ref = _run(torch, eng, vecs, None, tgt, resid=True, misfit=True)
    ref3 = _run(torch, eng, vecs[:3], None, tgt[:3], resid=True, misfit=True)
    assert eng.info("adj_tmem") == 0 and eng.info("last_adj_path") == 2
    eng.set_option("adj_cluster", 10)
    eng.set_option("adj_rows", rows)
    assert eng.info("adj_tmem") == 1 and eng.info("adj_cluster") == 10 and eng.info("cluster_adj") > 0
    out = _run(torch, eng, vecs, None, tgt, resid=True, misfit=True)
    eng.check()
    for a, b in zip(out, ref):
        assert np.array_equal(a, b)
    eng.set_option("adj_side", 4)                    # slots 16..19 of 20 tiled beside the clusters
    out3 = _run(torch, eng, vecs[:3], None, tgt[:3], resid=True, misfit=True)
    eng.check()
    assert eng.info("last_adj_side") == 0 or eng.info("last_adj_path") == 2
    for a, b in zip(out3, ref3):
        assert np.array_equal(a, b)
    eng.set_option("adj_side", 0)
    eng.set_option("test_skip_history_copy", 0)
    _run(torch, eng, vecs[:1], None, tgt[:1], resid=True)
    with pytest.raises(SeisError) as ei:
        eng.check()
    assert ei.value.status == -5
    eng.set_option("test_skip_history_copy", -1)
    again = _run(torch, eng, vecs, None, tgt, resid=True, misfit=True)
    eng.check()
    for a, b in zip(again, ref):
        assert np.array_equal(a, b)


def test_tensor_memory_forward_matches(torch):
    """The 10-CTA forward that keeps its band's alpha in tensor memory gives bitwise the
    records and the history (so the gradients) of the one that keeps it in shared memory,
    with and without the side forward beside it; the 16-CTA forward + tangent with alpha
    and dalpha in tensor memory gives bitwise the register version's records, tangent
    records and gradient."""
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=400)
    vecs, trues, _ = synthetic.batch(93, 4)
    eng = _engine(g, 4)
    eng.set_option("fwd_cluster", 10)
    assert eng.info("fwd_tmem") == 1                # the default where it applies
    eng.set_option("fwd_tmem", 0)
    tgt = _run(torch, eng, trues)[0]
    vd = np.random.default_rng(94).normal(0, 5.0, vecs.shape)
    ref = _run(torch, eng, vecs, None, tgt, resid=True, misfit=True)
    rec = _run(torch, eng, vecs)[0]
    ref_tan = _run(torch, eng, vecs, vd, tgt, resid=True)
    assert eng.info("fwd_tmem") == 0
    eng.set_option("fwd_tmem", 1)
    assert eng.info("fwd_tmem") == 1
    out_tan = _run(torch, eng, vecs, vd, tgt, resid=True)     # the forward + tangent with alpha, dalpha in TMEM
    for a, b in zip(out_tan, ref_tan):
        assert (a is None and b is None) or np.array_equal(a, b)
    for side in (0, 5):
        eng.set_option("fwd_side", side)
        out = _run(torch, eng, vecs, None, tgt, resid=True, misfit=True)
        eng.check()
        for a, b in zip(out, ref):
            assert np.array_equal(a, b)
        assert np.array_equal(_run(torch, eng, vecs)[0], rec)
        part = _run(torch, eng, vecs[:3], None, tgt[:3], resid=True, misfit=True)
        assert np.array_equal(part[2], ref[2][:3]) and np.array_equal(part[0], ref[0][:3])


def test_autotuner_picks_and_caches(torch, tmp_path):
    from seismic_gb300 import autotune
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=300)
    cache = str(tmp_path / "cfg.json")
    cands = [{"sweep_path": 1, "fwd_cluster": 8, "chunk": 0}, {"sweep_path": 2, "fwd_cluster": 8, "chunk": 0},
             {"sweep_path": 2, "fwd_cluster": 16, "chunk": 0},
             {"sweep_path": 2, "fwd_cluster": 8, "columns": 1, "chunk": 0}]
    best = autotune.tune(g, 2, cache_path=cache, cands=cands)
    assert best["sweep_path"] in (1, 2) and len(best["timings"]) == 4
    # chunks x (tiled, one or two steps per launch + 3 forward cluster sizes x (column pairs with the
    # 10- or 16-CTA adjoint, single columns with the 16-CTA adjoint))
    assert len(autotune.candidates(g, 64)) == 4 * (2 + 3 * 3)
    eng = autotune.Engine(g, max_models=64)
    sides = autotune.side_candidates(eng, {"sweep_path": 2, "fwd_cluster": 10, "columns": 2, "chunk": 0})
    assert any(c.get("adj_side") == 0 for c in sides) and any(c.get("adj_side", 0) > 0 for c in sides)
    assert any(c.get("fwd_side_cluster") == 8 and c["fwd_side"] == 34 for c in sides)   # the engine's split
    assert any(c.get("fwd_side_cluster") == 0 and c["fwd_side"] > 0 for c in sides)
    eng.close()
    again = autotune.tune(g, 2, cache_path=cache)            # from the cache, no re-timing
    assert again == best
    eng = autotune.tuned_engine(g, 2, cache_path=cache)
    assert eng.info("sweep_path") == best["sweep_path"]


def test_bounded_wait_reports_timeout_and_engine_recovers(torch):
    """A history copy that never arrives: the adjoint's bounded wait gives up, the
    device status reports the timeout, and the next call is correct again."""
    from seismic_gb300._lib import SeisError
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=200)
    vec = _model(3, 70, 70, "layered")
    w = np.random.default_rng(0).normal(0, 1e-2, g.nrecords)
    eng = _engine(g, 1, chunk=1)
    assert eng.info("cluster_adj") > 0
    good = _run(torch, eng, vec, None, w)
    eng.set_option("test_skip_history_copy", 0)      # level 0 is consumed at the last reverse step
    _run(torch, eng, vec, None, w)
    with pytest.raises(SeisError) as ei:
        eng.check()
    assert ei.value.status == -5
    eng.set_option("test_skip_history_copy", -1)
    again = _run(torch, eng, vec, None, w)
    eng.check()
    assert np.array_equal(again[2], good[2])


def test_fused_tiled_adjoint_steps_are_single_steps(torch):
    """Two reverse steps per launch give bitwise the one-step-per-launch gradient
    (odd nt: the last step runs alone), whole history and checkpointed."""
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=301)
    vecs, trues, _ = synthetic.batch(41, 2)
    w = np.random.default_rng(42).normal(0, 1e-2, (2, g.nrecords))
    eng = _engine(g, 2)
    eng.set_option("sweep_path", 1)
    fused = _run(torch, eng, vecs, None, w)
    eng.set_option("adj_fuse", 0)
    single = _run(torch, eng, vecs, None, w)
    assert np.array_equal(fused[2], single[2])
    eng.set_option("checkpoint_every", 25)
    ck_single = _run(torch, eng, vecs, None, w)
    eng.set_option("adj_fuse", 1)
    ck_fused = _run(torch, eng, vecs, None, w)
    assert np.array_equal(ck_fused[2], single[2]) and np.array_equal(ck_single[2], single[2])


@pytest.mark.parametrize("shape", [(70, 70), (100, 140)])
def test_fused_tiled_forward_steps_are_single_steps(torch, shape):
    """Two forward steps per launch give bitwise the one-step-per-launch records,
    tangent and gradient (odd nt: the last step runs alone), whole history and
    checkpointed (odd interval: pairs never cross a checkpoint)."""
    from seismic_gb300.geometry import Geometry
    nz, nx = shape
    g = Geometry.reference(nt=301) if shape == (70, 70) else \
        Geometry(nz=nz, nx=nx, nbc=120, nt=301, source_x_cells=(0, 47, 139), receiver_x_cells=tuple(range(0, 140, 3)))
    vecs = np.stack([_model(51, nz, nx), _model(52, nz, nx, "layered")])
    rng = np.random.default_rng(43)
    vd = rng.normal(0, 1.0, (2, g.nv))
    w = rng.normal(0, 1e-2, (2, g.nrecords))
    eng = _engine(g, 2)
    eng.set_option("sweep_path", 1)
    fused_rec = _run(torch, eng, vecs)
    assert eng.info("last_fwd_launches") == 151            # one chunk: 150 pairs and the last step
    fused = _run(torch, eng, vecs, None, w)
    fused_tan = _run(torch, eng, vecs, vd)
    eng.set_option("fwd_fuse", 0)
    single_rec = _run(torch, eng, vecs)
    assert eng.info("last_fwd_launches") == 301
    single = _run(torch, eng, vecs, None, w)
    single_tan = _run(torch, eng, vecs, vd)
    assert np.array_equal(fused_rec[0], single_rec[0])
    assert np.array_equal(fused[0], single[0]) and np.array_equal(fused[2], single[2])
    assert np.array_equal(fused_tan[1], single_tan[1]) and np.array_equal(fused_tan[0], single[0])
    eng.set_option("checkpoint_every", 25)
    ck_single = _run(torch, eng, vecs, None, w)
    eng.set_option("fwd_fuse", 1)
    ck_fused = _run(torch, eng, vecs, None, w)
    assert np.array_equal(ck_fused[2], single[2]) and np.array_equal(ck_single[2], single[2])
    assert np.array_equal(ck_fused[0], single[0])


@pytest.mark.parametrize("path", [0, 1])
def test_host_buffer_calls_match_device_calls(torch, path):
    """Inputs and outputs in host memory (pinned, pageable, NumPy): the engine stages
    the copies itself (targets uploaded during the forward sweep, records downloaded
    chunk by chunk during the adjoint sweep) and returns bitwise the device call's
    results; several chunks, the last one partial."""
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=301)
    vecs, trues, _ = synthetic.batch(61, 3)
    rng = np.random.default_rng(62)
    vd = rng.normal(0, 1.0, (3, g.nv))
    eng = _engine(g, 3, chunk=4)
    if path:
        eng.set_option("sweep_path", path)
    tgt = _run(torch, eng, trues)[0]
    dev = _run(torch, eng, vecs, vd, tgt, resid=True, misfit=True)
    pinned = lambda a: torch.as_tensor(np.asarray(a, np.float64)).pin_memory()
    pageable = lambda a: torch.as_tensor(np.array(a, np.float64))
    for conv in (pinned, pageable, lambda a: np.array(a, np.float64)):
        out = eng.vel_to_seis(conv(vecs), conv(vd), conv(tgt), adjoint_on_residual=True, want_misfit=True)
        for a, b in zip(out, dev):
            assert a.device.type == "cpu"
            assert np.array_equal(a.numpy(), b)
    # a host call between device calls leaves them unchanged
    again = _run(torch, eng, vecs, vd, tgt, resid=True, misfit=True)
    for a, b in zip(again, dev):
        assert np.array_equal(a, b)


def test_side_adjoint_matches_cluster_adjoint(torch):
    """Slots of a chunk whose adjoint runs on the tiled kernels beside the cluster
    adjoint (concurrently, on other streams) give bitwise the all-cluster gradient;
    full and partial chunks."""
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=301)
    vecs, trues, _ = synthetic.batch(71, 4)
    eng = _engine(g, 4)
    assert eng.info("cluster_adj") > 0
    tgt = _run(torch, eng, trues)[0]
    eng.set_option("adj_side", 0)
    ref = _run(torch, eng, vecs, None, tgt, resid=True, misfit=True)
    ref3 = _run(torch, eng, vecs[:3], None, tgt[:3], resid=True, misfit=True)
    assert eng.info("last_adj_side") == 0
    eng.set_option("adj_side", 6)                    # slots 14..19 of 20
    side = _run(torch, eng, vecs, None, tgt, resid=True, misfit=True)
    assert eng.info("last_adj_side") == 6 and eng.info("last_adj_path") == 2
    side3 = _run(torch, eng, vecs[:3], None, tgt[:3], resid=True, misfit=True)
    assert eng.info("last_adj_side") == 1            # 15 active slots: only slot 14 beside
    for a, b in zip(side, ref):
        assert np.array_equal(a, b)
    for a, b in zip(side3, ref3):
        assert np.array_equal(a, b)


def test_side_forward_matches_cluster_forward(torch):
    """Slots of a chunk whose forward (records only, with the history for a gradient,
    with the tangent) runs on the tiled kernels beside the cluster forward give
    bitwise the all-cluster results; full and partial chunks."""
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=301)
    vecs, trues, _ = synthetic.batch(81, 4)
    vd = np.random.default_rng(82).normal(0, 1.0, (4, g.nv))
    eng = _engine(g, 4)
    tgt = _run(torch, eng, trues)[0]
    eng.set_option("adj_side", 0)
    eng.set_option("fwd_side", 0)
    cases = [(vecs, None, None), (vecs, None, tgt), (vecs, vd, None), (vecs[:3], None, tgt[:3]),
             (vecs, vd, tgt)]
    ref = [_run(torch, eng, v, d, w, resid=w is not None) for v, d, w in cases]
    eng.set_option("fwd_side", 7)                    # slots 13..19 of 20
    # the side slots on the tiled kernels, and (automatic beside 10-CTA main clusters) on
    # two concurrent 8-CTA cluster sweeps; the tangent's side slots stay tiled
    for side_cluster in (0, -1):
        eng.set_option("fwd_side_cluster", side_cluster)
        assert eng.info("fwd_side_cluster") == (8 if side_cluster else 0)
        for (v, d, w), r in zip(cases, ref):
            out = _run(torch, eng, v, d, w, resid=w is not None)
            assert eng.info("last_fwd_side") == (7 if len(v) == 4 else 2)
            assert eng.info("last_fwd_path") == 2
            for a, b in zip(out, r):
                assert (a is None and b is None) or np.array_equal(a, b)


def test_forward_side_clusters_split_partial_chunks(torch):
    """The automatic forward side split runs on each chunk's own shot count: 8 models (40
    shots) in an engine of 160 slots put the shots beyond whole rounds of the main
    clusters on the 8-CTA side clusters; results bitwise those without side clusters."""
    import math
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference(nt=301)
    vecs, trues, _ = synthetic.batch(83, 8)
    eng = _engine(g, 32)
    tgt = _run(torch, eng, trues)[0]
    eng.set_option("fwd_side_cluster", 0)
    ref = _run(torch, eng, vecs, None, tgt, resid=True)
    eng.set_option("fwd_side_cluster", -1)
    out = _run(torch, eng, vecs, None, tgt, resid=True)
    ncl, best, side = eng.info("cluster_fwd10"), 1e30, 0
    for r in range(1, -(-40 // ncl) + 1):          # the engine's rule: max(main rounds, side rounds x 1.29)
        sd = max(0, 40 - r * ncl)
        t = max(r, math.ceil(sd / 2) * 1.29)
        if t < best:
            best, side = t, sd
    assert eng.info("last_fwd_side") == side
    # the adjoint's automatic (tiled) side split follows the chunk's 40 shots as well
    assert eng.info("last_adj_side") >= 1
    for a, b in zip(out, ref):
        assert (a is None and b is None) or np.array_equal(a, b)
    # and so does the tangent's (tiled side graphs captured per split)
    vd = np.random.default_rng(84).normal(0, 1.0, (8, g.nv))
    tan = _run(torch, eng, vecs, vd)
    assert eng.info("last_fwd_side") >= 1
    eng.set_option("fwd_side", 0)
    eng.set_option("adj_side", 0)
    tan0 = _run(torch, eng, vecs, vd)
    for a, b in zip(tan, tan0):
        assert (a is None and b is None) or np.array_equal(a, b)
    assert np.array_equal(_run(torch, eng, vecs, None, tgt, resid=True)[2], ref[2])


def test_benchmark_workload_batched_equals_alone(torch):
    """The benchmark workload at full size (64 models x 5 shots, 70x70, nt=1000, one
    chunk of 320 shots with the side sweeps): records, gradient and misfit of every
    model bitwise the same as the model alone (one shot per launch); the misfit is the
    FP64 sum of squared residuals of the returned records."""
    from seismic_gb300 import synthetic
    from seismic_gb300.geometry import Geometry
    import gc
    gc.collect()                                  # engines of earlier tests release their memory
    g = Geometry.reference(nt=1000)
    vecs, trues, _ = synthetic.batch(2024, 64)
    eng = _engine(g, 64)
    tgt = _run(torch, eng, trues)[0]
    full = _run(torch, eng, vecs, None, tgt, resid=True, misfit=True)
    if eng.slots == 320:                          # one chunk (the free HBM holds it on a GB300)
        assert eng.info("last_adj_side") > 0 and eng.info("last_fwd_side") > 0
    eng.close()
    one = _engine(g, 1, chunk=1)
    for m in range(64):
        r = _run(torch, one, vecs[m], None, tgt[m], resid=True, misfit=True)
        assert np.array_equal(full[0][m], r[0][0]) and np.array_equal(full[2][m], r[2][0])
        assert full[3][m] == r[3][0]
    one.close()
    resid = full[0] - tgt
    np.testing.assert_allclose(full[3], np.sum(resid * resid, axis=1), rtol=1e-12)


@pytest.mark.parametrize("geo", ["reference", "ragged"])
def test_tiled_adjoint_load_batching_is_bitwise(torch, geo):
    """The two-step tiled adjoint issues the history and gradient-sum loads of 1, 2 or 4
    rows of a thread together (adj_hoist): the same gradients and misfits bit for bit,
    including tiles whose last rows lie past the grid."""
    from seismic_gb300 import synthetic
    from seismic_gb300.engine import Engine
    from seismic_gb300.geometry import Geometry
    g = (Geometry.reference(nt=200) if geo == "reference"
         else Geometry(nz=37, nx=52, nbc=21, nt=220, source_x_cells=(3, 40), receiver_x_cells=tuple(range(0, 52, 3))))
    rng = np.random.default_rng(17)
    v = torch.as_tensor(np.stack([synthetic.to_vector(synthetic.model(rng, "faulted", g.nz, g.nx)) for _ in range(2)]),
                        device="cuda")
    w = torch.as_tensor(rng.normal(0, 1e-2, (2, g.nrecords)), device="cuda")
    eng = Engine(g, max_models=2)
    eng.set_option("sweep_path", 1)
    outs = []
    for h in (1, 2, 4):
        eng.set_option("adj_hoist", h)
        assert eng.info("adj_hoist") == h
        _, _, gr, mf = eng.vel_to_seis(v, None, w, adjoint_on_residual=True, want_misfit=True)
        torch.cuda.synchronize()
        eng.check()
        outs.append((gr.cpu(), mf.cpu()))
    assert all(torch.equal(o[0], outs[0][0]) and torch.equal(o[1], outs[0][1]) for o in outs[1:])
    with pytest.raises(Exception):
        eng.set_option("adj_hoist", 3)
    eng.close()
