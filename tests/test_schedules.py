"""Schedules, family dispatch and the result cache: host logic (no GPU)."""
import math

import numpy as np
import pytest
import torch

from seismic_gb300 import schedules as S
from seismic_gb300 import synthetic
from seismic_gb300.data import Seismogram, Velocity


def _vel(v):
    v = torch.as_tensor(np.asarray(v, np.float64))
    return Velocity(data=v, min_vel=v.min())


def test_kpi_flatvel_symmetric_records():
    rng = np.random.default_rng(0)
    half = rng.normal(size=(999, 70))
    seis = np.stack([half, rng.normal(size=(999, 70)), rng.normal(size=(999, 70)),
                     rng.normal(size=(999, 70)), half[:, ::-1]])
    assert S.kpi_flatvel(seis) == 0.0
    seis[4, 10, 3] += 1.0
    assert S.kpi_flatvel(seis) == pytest.approx(math.sqrt(1.0 / (999 * 70)))


def test_kpi_style_b_and_fault_a():
    v = np.full((70, 70), 3000.0)
    v[:, :35] = 2000.0
    assert S.kpi_style_b(v) == 2450               # two values, 35 columns each
    assert S.kpi_fault_a(v) == 4900               # two flat components cover everything
    v2 = v.copy()
    v2[0, 0] = 4500.0                             # a third (single-cell) component
    assert S.kpi_fault_a(v2) == 4899
    g = np.arange(4900, dtype=np.float64).reshape(70, 70) * 0.4   # smooth ramp, steps 0.4 / 28 m/s
    assert S.kpi_style_b(g) <= 8
    assert S.kpi_fault_a(g) == 140                # rows are the components (vertical steps 28 > 10)


def test_kpi_style_a_quadratic_form():
    rng = np.random.default_rng(1)
    vec = rng.normal(size=4901)
    Pm = np.diag(rng.uniform(0.5, 2.0, 4900))
    assert S.kpi_style_a(vec, Pm) == pytest.approx(float(vec[:-1] @ Pm @ vec[:-1]))


def test_result_cache_round_trip(tmp_path):
    cache = S.ResultCache(str(tmp_path))
    s = S.Sample(seismogram=Seismogram(filename="/data/x/seis2_1_0.npy", ind=7), family="FlatVelA")
    assert s.cache_name() == "seis2_1_0__FlatVelA__7"
    assert cache.get("TV2D", s) is None
    v = _vel(np.arange(4900.0).reshape(70, 70))
    cache.put("TV2D", s, v)
    got = cache.get("TV2D", s)
    assert torch.equal(got.data, v.data) and float(got.min_vel) == 0.0
    s2 = S.Sample(seismogram=Seismogram(data=torch.zeros(5, 999, 70)), name="synthetic3")
    assert s2.cache_name() == "synthetic3__test"


def test_schedule_settings_are_the_reference_ones():
    """Stage settings of core/seis_model.py:15-138 (full and test_mode values)."""
    fv = S.flat_vel(device="cpu")
    assert (type(fv.prior).__name__, fv.prior.lam, fv.prior.epsilon, fv.maxiter) == ("RowTotalVariation", 1e-8, 0.1, 1000)
    assert (fv.lbfgs_tolerance_change, fv.lbfgs_tolerance_grad, fv.round_results) == (1e-9, 1e-7, True)
    assert S.flat_vel(True, "cpu").maxiter == 30

    sa = S.style_a(device="cpu")
    p = sa.stages[0].prior
    assert (p.transform, p.svd_cutoff, p.lam, sa.stages[0].maxiter) == (True, 1.0, 1e-12, 2500)
    assert sa.stages[0].lbfgs_tolerance_grad == 10 ** 6.5
    assert (sa.stages[1].maxiter, sa.stages[1].cache_name) == (0, "Style_A_refine")
    assert S.style_a(True, "cpu").stages[0].prior.svd_cutoff == 10000.0

    sb = S.style_b(device="cpu")
    p = sb.stages[0].prior
    assert (p.length_scale, p.sigma, p.noise, p.sigma_mean, p.sigma_slope, p.transform, p.lam) == \
        (1.96, 158.0, 58.0, 1239.0, 92.0, False, 1e-15)
    assert (sb.stages[0].maxiter, sb.stages[1].maxiter, sb.stages[1].seis_error_tolerance) == (1500, 7500, 2.5e-9)

    t = S.tv2d(device="cpu")
    assert [st.maxiter for st in t.stages] == [2500, 10000, 1500]
    assert [st.lbfgs_tolerance_grad for st in t.stages] == [10 ** 3.5, 10 ** 3.5, 10 ** 2.5]
    assert (t.stages[0].prior.lam, t.round_results) == (1e-8, True)
    p3 = t.stages[2].prior
    assert type(p3).__name__ == "RestrictFlatAreas" and p3.diff_threshold == 1.0
    assert p3.underlying_prior.lam == pytest.approx(1e-9)
    assert [st.maxiter for st in S.tv2d(True, "cpu").stages] == [75, 5, 10]

    te = S.tv2d_easy(device="cpu")
    assert (te.prior.lam, te.lbfgs_tolerance_grad, te.maxiter, te.round_results) == \
        (1e-7, pytest.approx(10 ** 4.5), 600, True)


def test_family_split_routing():
    fs = S.FamilySplit(device="cpu")
    fs.style_a_precision = np.zeros((4900, 4900))     # every model "likely" under Style A
    rng = np.random.default_rng(2)
    half = rng.normal(size=(999, 70))
    sym = torch.as_tensor(np.stack([half, half, half, half, half[:, ::-1]]))
    asym = torch.as_tensor(rng.normal(size=(5, 999, 70)))
    v = _vel(synthetic.layered(rng))
    assert fs.classify(S.Sample(Seismogram(data=sym), v)) == "FlatVel"
    assert fs.classify(S.Sample(Seismogram(data=asym), v)) == "Style_A"
    fs.style_a_precision = np.eye(4900)                # |v|^2 ~ 1e10 > e^13: not Style A
    smooth = _vel(1500.0 + np.add.outer(np.arange(70) * 40.0, np.arange(70) * 0.5))
    assert fs.classify(S.Sample(Seismogram(data=asym), smooth)) == "Style_B"
    two = np.full((70, 70), 3000.0)
    two[40:, :] = 4000.0
    assert fs.classify(S.Sample(Seismogram(data=asym), _vel(two))) == "TV2Deasy"
    many = np.zeros((70, 70))
    for k in range(7):
        many[10 * k:10 * k + 10, :] = 1500.0 + 400.0 * k
    assert fs.classify(S.Sample(Seismogram(data=asym), _vel(many))) == "TV2D"
