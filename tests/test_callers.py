"""The reference's callers of the engine, restated: priors (CPU, against the
reference's own values) and the L-BFGS pieces that need no GPU."""
import numpy as np
import pytest
import torch

from conftest import load_golden, rel_l2


@pytest.fixture(scope="module")
def gold():
    return load_golden("callers")


def _t(a):
    return torch.as_tensor(np.asarray(a), dtype=torch.float64)


@pytest.mark.parametrize("name,cls", [("rowtv", "RowTotalVariation"), ("tv", "TotalVariation"),
                                      ("se", "SquaredExponential")])
def test_priors_match_reference(gold, name, cls):
    from seismic_gb300 import priors
    pr = getattr(priors, cls)(70, 70, device="cpu")
    pr.lam = 1.0
    pr.prep()
    c, g = pr.compute_cost_and_gradient(_t(gold[f"{name}_x"]), compute_gradient=True)
    # the SE precision matrix inverts a covariance of condition number ~2e11 (its constant
    # and depth-slope terms): two correct inverses differ by up to cond * eps ~ 2e-5 there
    tol = 1e-4 if name == "se" else 1e-12
    assert abs(float(c) / float(gold[f"{name}_cost"]) - 1) < tol
    assert rel_l2(g.numpy(), gold[f"{name}_grad"]) < max(tol, 1e-10)


def test_squared_exponential_svd_basis_matches_reference(gold):
    from seismic_gb300 import priors
    pr = priors.SquaredExponential(70, 70, device="cpu", transform=True, svd_cutoff=1.0)
    pr.lam = 1.0
    pr.prep()
    assert pr.N == int(gold["se_svd_N"])
    assert rel_l2(torch.linalg.norm(pr.basis_vectors, dim=0).numpy(), gold["se_svd_basis_colnorms"]) < 1e-8
    c, g = pr.compute_cost_and_gradient(_t(gold["se_svd_x"]), compute_gradient=True)
    assert abs(float(c) / float(gold["se_svd_cost"]) - 1) < 1e-12
    assert rel_l2(g.numpy(), gold["se_svd_grad"]) < 1e-12


def test_restrict_flat_areas_matches_reference(gold):
    from seismic_gb300 import priors
    under = priors.TotalVariation(70, 70, device="cpu")
    under.lam = 1.0
    pr = priors.RestrictFlatAreas(under)
    pr.prep()
    pr.adapt(gold["rfa_vel"])
    assert pr.N == int(gold["rfa_N"])
    c, g = pr.compute_cost_and_gradient(_t(gold["rfa_x"]), compute_gradient=True)
    assert abs(float(c) / float(gold["rfa_cost"]) - 1) < 1e-12
    assert rel_l2(g.numpy(), gold["rfa_grad"]) < 1e-10


@pytest.mark.parametrize("cls", ["RowTotalVariation", "TotalVariation", "SquaredExponential"])
def test_prior_gradient_finite_difference_any_grid(cls):
    """Directional derivative with offset 1e-6 N(0,1), rel < 1e-6 (core/seis_test.py:48-69), on a 23x31 grid."""
    from seismic_gb300 import priors
    pr = getattr(priors, cls)(23, 31, device="cpu")
    pr.lam = 15.0
    pr.prep()
    base = torch.as_tensor(np.random.default_rng(0).normal(0, 1, (pr.N, 1)))
    off = 1e-6 * torch.as_tensor(np.random.default_rng(0).normal(0, 1, (pr.N, 1)))
    c, g = pr.compute_cost_and_gradient(base, compute_gradient=True)
    c2 = pr.compute_cost_and_gradient(base + off)
    assert abs(float((g * off).sum()) - float(c2 - c)) / abs(float(c2 - c)) < 1e-6


def test_cubic_interpolate_minimum():
    from seismic_gb300.numerics import cubic_interpolate
    # f(t) = (t - 0.3)^2: exact minimiser from two points with slopes
    t = cubic_interpolate(0.0, 0.09, -0.6, 1.0, 0.49, 1.4)
    assert abs(t - 0.3) < 1e-12
    # no real minimiser (d1^2 < g1 g2): the middle of the bounds
    assert cubic_interpolate(0.0, 0.0, 3.0, 1.0, 2.0, 3.0, bounds=(0.2, 0.8)) == 0.5
