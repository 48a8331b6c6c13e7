"""CPU: host-side logic -- geometry, synthetic models, the C ABI's exports."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def test_reference_geometry_indices():
    """Geometry.reference() gives the reference's padded indices (core/seis_forward2.py:86-101):
    sources at row 121, columns 120+{0,17,34,52,69}; receivers row 121, columns 120..189."""
    from seismic_gb300.geometry import Geometry
    g = Geometry.reference()
    assert list(g.src_z) == [121] * 5
    assert list(g.src_x) == [120, 137, 154, 172, 189]
    assert list(g.rec_z) == [121] * 70 and list(g.rec_x) == list(range(120, 190))
    assert g.nv == 4901 and g.nrecords == 5 * 999 * 70 and g.padded_shape == (310, 310)
    assert list(g.src_z * 310 + g.src_x) == [121 * 310 + 120 + c for c in (0, 17, 34, 52, 69)]


def test_geometry_matches_oracle_geometry():
    from oracle.oracle import OracleGeometry
    from seismic_gb300.geometry import Geometry
    for kw in [dict(), dict(nz=100, nx=140, nt=1500, source_x_cells=(0, 46, 93, 139)),
               dict(nz=12, nx=9, nbc=4, source_z_cell=0, receiver_z_cell=0, source_x_cells=(0, 8))]:
        g = Geometry(**kw)
        o = OracleGeometry(**{("src_x_cells" if k == "source_x_cells" else
                               "src_z_cells" if k == "source_z_cell" else
                               "rec_z_cells" if k == "receiver_z_cell" else k): v for k, v in kw.items()})
        for a in ("src_z", "src_x", "rec_z", "rec_x"):
            assert np.array_equal(getattr(g, a), getattr(o, a)), a


def test_surface_geometry_spreads_shots():
    from seismic_gb300.geometry import Geometry
    assert Geometry.surface(70, 70, 5, 1000).source_x_cells == (0, 17, 34, 52, 69)
    g = Geometry.surface(200, 300, 20, 2000)
    assert g.nshots == 20 and g.src_x[0] == 120 and g.src_x[-1] == 120 + 299
    with pytest.raises(ValueError):
        Geometry(nbc=1)


@pytest.mark.parametrize("family", ["layered", "faulted", "curved"])
def test_synthetic_models(family):
    from seismic_gb300 import synthetic
    a = synthetic.model(np.random.default_rng(3), family, 70, 70)
    b = synthetic.model(np.random.default_rng(3), family, 70, 70)
    assert np.array_equal(a, b) and a.shape == (70, 70)
    assert a.min() >= 1500 and a.max() <= 4500
    vec = synthetic.to_vector(a)
    assert vec.shape == (4901,) and vec[-1] == a.min()
    if family == "layered":
        assert np.all(np.diff(a[:, 0]) >= 0)


def test_synthetic_batch_and_perturbation():
    from seismic_gb300 import synthetic
    vecs, trues, fams = synthetic.batch(7, 6)
    assert vecs.shape == (6, 4901) and fams[:3] == ["layered", "faulted", "curved"]
    r = trues[:, :-1] / vecs[:, :-1] - 1
    assert np.abs(r).max() <= 0.05 + 1e-12 and np.abs(r).max() > 0.01


def _header_functions():
    src = open(os.path.join(ROOT, "include", "seis_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(seis_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_header_symbol():
    """The C-ABI library builds for sm_103a and exports each function the header declares
    (loading it makes no CUDA call)."""
    from seismic_gb300 import _lib
    path = _lib.build()
    lib = ctypes.CDLL(path)
    names = _header_functions()
    assert "seis_vel_to_seis" in names and "seis_create" in names
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) <= set(_lib.EXPORTS), set(names) - set(_lib.EXPORTS)


def test_create_rejects_bad_geometry_without_gpu():
    """Argument validation happens before any CUDA call."""
    from seismic_gb300 import _lib
    from seismic_gb300.geometry import Geometry
    lib = _lib.load()
    g, keep = Geometry.reference().to_c()
    h = ctypes.c_void_p()
    assert lib.seis_create(ctypes.byref(g), 0, 0, ctypes.byref(h)) == -1
    assert b"max_models" in lib.seis_last_error(None)
    g.nt = 100  # shorter than the 147-tap Ricker wavelet
    assert lib.seis_create(ctypes.byref(g), 1, 0, ctypes.byref(h)) == -1
    assert b"Ricker" in lib.seis_last_error(None)
    g.nt = 999
    g.nbc = 1
    assert lib.seis_create(ctypes.byref(g), 1, 0, ctypes.byref(h)) == -1
    del keep


def test_all_shots_workspace_checkpoints_largest_histories_first():
    """The one-launch uneven batch sizes each set-up for all its shots: whole histories
    while they fit, then checkpointed adjoints for the largest history per shot first."""
    from seismic_gb300.geometry import Geometry
    from seismic_gb300.serving import all_shots_workspace, shot_workspace_bytes
    small = Geometry.surface(70, 70, 5, 1000)
    mid = Geometry.surface(200, 300, 10, 1500)
    big = Geometry.surface(350, 500, 10, 2000)
    setups = {"s": (small, 4), "m": (mid, 2), "b": (big, 1)}
    whole = {k: m * g.nshots * shot_workspace_bytes(g, 0) for k, (g, m) in setups.items()}
    plan = all_shots_workspace(setups, sum(whole.values()) + 1, 50)
    assert all(plan[k] == (0, whole[k]) for k in setups)
    # room for everything but the largest history: only the 350x500 set-up is checkpointed
    plan = all_shots_workspace(setups, whole["s"] + whole["m"] + 0.5 * whole["b"], 50)
    assert plan["b"][0] == 50 and plan["m"][0] == 0 and plan["s"][0] == 0
    assert plan["b"][1] == 10 * shot_workspace_bytes(big, 50) < whole["b"]
    # nothing fits whole: every set-up checkpointed, largest first
    plan = all_shots_workspace(setups, 1.0, 50)
    assert all(plan[k][0] == 50 for k in setups)


def test_concurrent_workspace_keeps_whole_histories_where_they_cost_the_most():
    """The concurrent uneven batch: each set-up's chunk fills the GPU on its own; whole
    histories while the minimum chunks fit, then checkpointed adjoints first where they
    free the most memory per unit of recomputed work (a set-up whose adjoint runs on
    clusters last); spare memory grows the chunks."""
    import math
    from seismic_gb300.geometry import Geometry
    from seismic_gb300.serving import concurrent_workspace, shot_workspace_bytes
    small = Geometry.surface(70, 70, 5, 2000)            # cluster adjoint, 13 resident clusters
    big = Geometry.surface(350, 500, 10, 2000)           # 590 x 740 padded: 228 tiles, tiled adjoint
    few = Geometry.surface(350, 500, 5, 1000)
    # (geometry, models, shots that fill the GPU, adjoint on clusters): 13 resident clusters
    # for 70x70; one wave of 608 tiled blocks over 228 tiles for 350x500
    fb = math.ceil(608 / 228)
    setups = {"s": (small, 2, 13, True), "b": (big, 4, fb, False), "f": (few, 1, fb, False)}
    fill = {"s": 10, "b": fb, "f": fb}                      # at most the set-up's shots
    whole = {k: fill[k] * shot_workspace_bytes(setups[k][0], 0) for k in setups}
    plan = concurrent_workspace(setups, sum(whole.values()), 50)
    assert {k: v for k, v in plan.items()} == {k: (0, fill[k]) for k in setups}
    # spare memory grows the chunks by work, up to each set-up's shots
    plan = concurrent_workspace(setups, 100 * sum(whole.values()), 50)
    assert plan == {"s": (0, 10), "b": (0, 40), "f": (0, 5)}
    # short of room for one: the set-up with the least work per byte (5 shots of nt 1000)
    # is checkpointed, the 40-shot set-up and the cluster one keep whole histories
    plan = concurrent_workspace(setups, sum(whole.values()) - 1, 50)
    assert plan["f"][0] == 50 and plan["b"][0] == 0 and plan["s"][0] == 0
    assert all(plan[k][1] >= fill[k] for k in setups)
    # two set-ups alike but for the adjoint's path (a 13-shot chunk either way): the
    # tiled one is checkpointed first
    two = {"c": (small, 4, 13, True), "t": (small, 4, 13, False)}
    w13, c13 = 13 * shot_workspace_bytes(small, 0), 13 * shot_workspace_bytes(small, 50)
    assert concurrent_workspace(two, w13 + c13, 50) == {"c": (0, 13), "t": (50, 13)}
    # nothing fits: every set-up checkpointed
    plan = concurrent_workspace(setups, 1.0, 50)
    assert all(plan[k] == (50, fill[k]) for k in setups)


def test_server_keeps_whole_histories_where_a_gpu_filling_chunk_fits(monkeypatch):
    """The inversion server checkpoints a grid only when a chunk of shots that fills the
    GPU does not fit its engine's share of the budget, and a request's footprint counts
    the shots its engine holds at once (not all of its shots)."""
    from seismic_gb300 import serving
    from seismic_gb300.geometry import Geometry
    from seismic_gb300.serving import InversionRequest, InversionServer, shot_workspace_bytes
    monkeypatch.setattr(serving, "fill_shots", lambda g, device: (3, False))
    big = Geometry.surface(350, 500, 20, 2000)
    W, C = shot_workspace_bytes(big, 0), shot_workspace_bytes(big, 50)

    class Prior:
        N = 10

    req = InversionRequest(rid=0, geometry=big, target=None, start=None, prior=Prior(), maxiter=10)
    # 8 engines (4 geometries x 2 lanes): each gets an eighth of the budget
    roomy = InversionServer(hbm_budget_bytes=8 * 5 * W, device=0)
    assert roomy._engine_share() == 5 * W and roomy._ck_for(big) == 0
    opt = serving.request_footprint(req, 0, 0)               # no shots: optimiser state, records, vectors
    assert roomy.footprint(req) == opt + 5 * W                # 5 of the 20 shots held at once
    tight = InversionServer(hbm_budget_bytes=8 * 2 * W, device=0)
    assert tight._ck_for(big) == 50                           # 3 whole-history shots do not fit
    assert tight.footprint(req) == serving.request_footprint(req, 50, (2 * W) // C)
    fixed = InversionServer(hbm_budget_bytes=8 * 5 * W, device=0, checkpoint_above_bytes=1 << 30)
    assert fixed._ck_for(big) == 50                           # the fixed rule: above 1 GiB per shot


def test_bench_roofline_follows_from_the_profile_summaries():
    """The bench line's roofline of the dominant cluster kernel: shared-memory wavefronts
    per point-step, DRAM bytes per point-step and the FMA-pipe fraction come from its ncu
    summary under profiles/; the peak is 128 B per clock per SM at the sampled clock."""
    import bench
    prof = bench.load_profile("adj_cluster_tm_kernel")
    assert prof["file"].startswith("profiles/") and prof["smem_wavefronts_per_point_step"] > 0
    ps, t = 2.99832e10, 40.99e-3                 # point-steps per launch, launch time of the benchmark
    r = bench.kernel_roofline("adj_cluster_tm_kernel", ps, 24 * ps, t, {"sm_mhz": 2070.0}, 152, 130)
    peak = 128 * 152 * 2070e6 / 1e9
    assert r["bound"] == "smem" and abs(r["peak"] - peak) < 1e-6
    assert abs(r["achieved"] - prof["smem_wavefronts_per_point_step"] * 128 * ps / t / 1e9) < 1e-6
    assert abs(r["frac"] - r["achieved"] / peak) < 1e-12
    assert abs(r["frac_on_busy_sms"] - r["frac"] * 152 / 130) < 1e-12
    assert r["traffic"] == prof["dram_bytes_per_point_step"] * ps
    assert r["fp32_issue_frac"] == prof["fma_pipe_active"]
    assert r["effective_hbm"]["frac"] > 1          # the algorithmic bytes never reach HBM
    # a tiled kernel streams through HBM: bound hbm against the measured copy bandwidth
    rt = bench.kernel_roofline("adj_step2_kernel", 1e9, 24e9, 10e-3, {}, 152, 152)
    assert rt["bound"] == "hbm" and abs(rt["frac"] - 24e9 / 10e-3 / 1e9 / rt["peak"]) < 1e-12
