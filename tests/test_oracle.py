"""CPU: the FP64 oracle against the reference's golden vectors and the
reference's own property tests (core/seis_test.py:16-46), re-hosted on
synthetic models."""
import numpy as np
import pytest

from conftest import load_golden, rel_l2

GOLDEN_CASES = ["ref70_layered", "ref70_faulted_residual"]


def _regen_inputs(gd, nv, nrecords):
    vec = gd["vec"][:, None]
    w = np.random.default_rng(int(gd["adjoint_seed"])).normal(0.0, float(gd["adjoint_sigma"]), (nrecords, 1))
    vd = None
    if "tangent_seed" in gd:
        vd = np.random.default_rng(int(gd["tangent_seed"])).normal(0.0, 1.0, (nv, 1))
    return vec, vd, w


def _rows_match(rec, row_sum, row_sumsq, tol):
    """Every (shot, time step) record row: its sum within tol of the row's absolute sum,
    its sum of squares within tol relative (rows that are zero in the reference stay zero)."""
    s, q, a = rec.sum(axis=2), (rec ** 2).sum(axis=2), np.abs(rec).sum(axis=2)
    nz = row_sumsq > 0
    return (np.all(np.abs(s - row_sum) <= tol * a) and np.all(q[~nz] == 0)
            and np.all(np.abs(q[nz] / row_sumsq[nz] - 1) < tol))


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_matches_reference_golden(oracle, case):
    """The C restatement reproduces the reference run (NumPy in place of CuPy) at
    the reference geometry: records to rounding, tangent and gradient to 1e-12."""
    gd = load_golden(case)
    g = oracle.OracleGeometry()
    vec, vd, w = _regen_inputs(gd, 4901, 349650)
    res, rd, ra = oracle.vel_to_seis(g, vec, vd, w, adjoint_on_residual=bool(gd["adjoint_on_residual"]))
    stride = int(gd["row_stride"])
    rec = res.reshape(5, 999, 70)
    assert rel_l2(rec[:, ::stride, :], gd["rec_rows"]) < 1e-13
    assert abs(res.sum() - gd["rec_sum"]) <= 1e-12 * np.abs(res).sum()
    assert abs((res ** 2).sum() / gd["rec_sumsq"] - 1) < 1e-12
    # every row, not only the stored tenth: the reference's per-row moments, which catch a
    # mistake planted in one value of a row the stored tenth leaves out
    assert _rows_match(rec, gd["rec_row_sum"], gd["rec_row_sumsq"], 1e-13)
    bad = rec.copy()
    bad[2, 501, int(np.argmax(np.abs(rec[2, 501])))] *= 1 + 1e-6
    assert rel_l2(bad[:, ::stride, :], gd["rec_rows"]) < 1e-13
    assert not _rows_match(bad, gd["rec_row_sum"], gd["rec_row_sumsq"], 1e-13)
    assert rel_l2(ra[:, 0], gd["grad"]) < 1e-12
    if vd is not None:
        drec = rd.reshape(5, 999, 70)
        assert rel_l2(drec[:, ::stride, :], gd["drec_rows"]) < 1e-12
        assert abs((rd ** 2).sum() / gd["drec_sumsq"] - 1) < 1e-12
        assert _rows_match(drec, gd["drec_row_sum"], gd["drec_row_sumsq"], 1e-10)


def _small_geometry(oracle, nt=300):
    return oracle.OracleGeometry(nz=24, nx=30, nbc=16, nt=nt, src_x_cells=(0, 11, 29))


def _small_model(seed, nz=24, nx=30):
    from seismic_gb300 import synthetic
    v = synthetic.model(np.random.default_rng(seed), "faulted", nz, nx)
    return synthetic.to_vector(v)[:, None]


def test_oracle_adjoint_dot_product(oracle):
    """<F(v)-w, J d> = <J^T (F(v)-w), d>, rel < 1e-10 (core/seis_test.py:26-38)."""
    g = _small_geometry(oracle)
    vec = _small_model(1)
    rng = np.random.default_rng(0)
    d = 1e-4 * rng.normal(0, 1, vec.shape) * 1000
    res0, _, _ = oracle.vel_to_seis(g, vec)
    w = res0 + rng.normal(0, 1, res0.shape) * np.abs(res0).max() * 0.1
    res, rd, ra = oracle.vel_to_seis(g, vec, d, w, adjoint_on_residual=True)
    r1 = np.sum((res - w) * rd)
    r2 = np.sum(ra * d)
    assert abs(r1 - r2) / abs(r1) < 1e-10


def test_oracle_tangent_vs_finite_difference(oracle):
    """rms(F(v+d)-F(v)-J d)/rms(F(v+d)-F(v)) < 1e-5 with d = 1e-4 N(0,1)
    (core/seis_test.py:41-44)."""
    g = _small_geometry(oracle)
    vec = _small_model(2)
    d = 1e-4 * np.random.default_rng(0).normal(0, 1, vec.shape)
    res, rd, _ = oracle.vel_to_seis(g, vec, d)
    res_off, _, _ = oracle.vel_to_seis(g, vec + d)
    num = np.sqrt(np.mean((res_off - res - rd) ** 2))
    den = np.sqrt(np.mean((res_off - res) ** 2))
    assert num / den < 1e-5


def test_oracle_gradient_vs_central_difference(oracle):
    """Gradient of 0.5*||F(v)-t||^2 against central differences along random directions."""
    g = _small_geometry(oracle, nt=200)
    vec = _small_model(3)
    t, _, _ = oracle.vel_to_seis(g, _small_model(4))
    _, _, grad = oracle.vel_to_seis(g, vec, None, t, adjoint_on_residual=True)
    rng = np.random.default_rng(5)
    for _ in range(3):
        d = rng.normal(0, 1, vec.shape)
        eps = 1e-3
        fp = 0.5 * np.sum((oracle.vel_to_seis(g, vec + eps * d)[0] - t) ** 2)
        fm = 0.5 * np.sum((oracle.vel_to_seis(g, vec - eps * d)[0] - t) ** 2)
        fd = (fp - fm) / (2 * eps)
        an = float(np.sum(grad * d))
        assert abs(fd - an) / abs(an) < 1e-6


def test_oracle_ricker_and_damp():
    from oracle import oracle as orc
    w = orc.ricker(15.0, 1e-3, 999)
    # nw = 147 taps centred on tap 74 (index 73) with peak 1
    assert np.argmax(w) == 73 and w[73] == 1.0 and np.all(w[147:] == 0) and w[146] != 0
    d = orc.damp(310, 310, 120, 10.0)
    # rows/columns 120..189 are the model; 150 is interior, 5 and 300 are in the bands
    assert d[150, 150] == 0.0 and d[0, 150] > 0 and d[150, 0] > 0 and d[300, 150] > 0
    assert d[5, 150] == d[150, 5] and d[5, 119] == 0.0 and d[0, 0] == d[150, 0]
    # corners take the x profile only (AbcCoef2D loop order, core/seis_forward2.py:53-58)
    assert d[5, 100] == d[150, 100] and d[5, 100] < d[5, 150]
    with pytest.raises(ValueError):
        orc.ricker(15.0, 1e-3, 100)


def test_oracle_nt_generalisation(oracle):
    """Records for nt=1000 extend the nt=999 records unchanged (causality)."""
    g1 = oracle.OracleGeometry(nz=16, nx=20, nbc=12, nt=180, src_x_cells=(3, 15))
    g2 = oracle.OracleGeometry(nz=16, nx=20, nbc=12, nt=181, src_x_cells=(3, 15))
    vec = _small_model(7, 16, 20)
    r1 = oracle.vel_to_seis(g1, vec)[0].reshape(2, 180, 20)
    r2 = oracle.vel_to_seis(g2, vec)[0].reshape(2, 181, 20)
    assert np.array_equal(r1, r2[:, :180])


def test_batch_calls_match_single_calls(oracle):
    """The threaded batch entry points (the CPU baseline's) give each model's single-call
    records and gradient bitwise."""
    g = _small_geometry(oracle, nt=200)
    vecs = np.stack([_small_model(s)[:, 0] for s in (3, 4, 5)])
    nr = g.nshots * g.nt * g.nrec
    res = oracle.batch_forward(g, vecs, 3)
    tg = res + np.random.default_rng(6).normal(0.0, 1e-3, res.shape)
    res2, grads = oracle.batch_cost_gradient(g, vecs, tg, 2)
    for i in range(3):
        r1, _, ra = oracle.vel_to_seis(g, vecs[i], None, tg[i], adjoint_on_residual=True)
        assert np.array_equal(res[i], r1[:, 0]) and np.array_equal(res2[i], r1[:, 0])
        assert np.array_equal(grads[i], ra[:, 0])
    assert res.shape == (3, nr)
