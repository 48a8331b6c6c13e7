"""GPU parity at the larger grids of the uneven-batch workload: the CUDA engine,
through the C ABI, against the FP64 oracle on 100x140 (nt 1000), 200x300
(nt 1500) and 350x500 (nt 2000) models -- padded 340x380, 440x540 and 590x740,
all wider than the cluster kernels' 316 columns, so these run the tiled
two-step sweeps.  Records, tangent records, misfit and gradient, on the default
path (whole forward history) and with checkpointed adjoints
(``checkpoint_every`` = 50, which must give bitwise the same gradient).

The reference hard-codes its 70x70 geometry (core/seis_forward2.py:69-101); the
oracle restates its discretisation for any grid (pinned to the reference's own
output at 70x70 in test_oracle.py), so these grids are pinned through it.

Tolerances (relative L2, FP32 sweeps against FP64): records <= 1e-5, tangent
records and gradients <= 1e-4, misfit <= 1e-5.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

REC_TOL = 1e-5
TAN_TOL = 1e-4
GRAD_TOL = 1e-4
MISFIT_TOL = 1e-5

LARGE = [
    # name, nz, nx, shots, nt, family
    ("100x140", 100, 140, 5, 1000, "curved"),
    ("200x300", 200, 300, 10, 1500, "faulted"),
    ("350x500", 350, 500, 3, 2000, "layered"),
]


@pytest.mark.parametrize("name,nz,nx,ns,nt,family", LARGE, ids=[c[0] for c in LARGE])
def test_large_grid_vs_oracle(oracle, parity_report, name, nz, nx, ns, nt, family):
    import torch

    from seismic_gb300 import synthetic
    from seismic_gb300.engine import Engine
    from seismic_gb300.geometry import Geometry
    assert torch.cuda.is_available()
    g = Geometry.surface(nz, nx, ns, nt)
    assert g.cfl(4500.0) <= 0.5
    rng = np.random.default_rng(1000 + nz)
    v = synthetic.model(rng, family, nz, nx)
    vec = synthetic.to_vector(v)
    vt = synthetic.to_vector(synthetic.perturbed(rng, v))
    vd = rng.normal(0.0, 10.0, g.nv)
    tgt = oracle.vel_to_seis(g, vt[:, None])[0][:, 0]
    o_res, o_rd, o_ra = oracle.vel_to_seis(g, vec[:, None], vd[:, None], tgt[:, None], adjoint_on_residual=True)
    o_mf = float(np.sum((o_res[:, 0] - tgt) ** 2))

    eng = Engine(g, max_models=1)
    dev = lambda a: torch.as_tensor(a[None, :], device="cuda")
    res, rd, ra, mf = eng.vel_to_seis(dev(vec), dev(vd), dev(tgt), adjoint_on_residual=True, want_misfit=True)
    torch.cuda.synchronize()
    eng.check()
    # 100x140 (row pitch 384) has cluster sweeps but no forward + tangent cluster shape: its
    # adjoint runs on clusters; the wider grids run tiled sweeps
    cl = name == "100x140"
    assert eng.info("last_fwd_path") == 1 and eng.info("last_adj_path") == (2 if cl else 1)
    errs = dict(records=rel_l2(res.cpu().numpy()[0], o_res), tangent=rel_l2(rd.cpu().numpy()[0], o_rd),
                gradient=rel_l2(ra.cpu().numpy()[0], o_ra), misfit=abs(float(mf[0]) / o_mf - 1.0))
    # without the tangent the forward takes the cluster path too: bitwise the tiled records
    res2, _, ra2, mf2 = eng.vel_to_seis(dev(vec), None, dev(tgt), adjoint_on_residual=True, want_misfit=True)
    torch.cuda.synchronize()
    eng.check()
    assert eng.info("last_fwd_path") == (2 if cl else 1)
    assert torch.equal(res2, res) and torch.equal(ra2, ra) and torch.equal(mf2, mf)
    eng.set_option("checkpoint_every", 50)
    _, _, ra_ck, mf_ck = eng.vel_to_seis(dev(vec), None, dev(tgt), adjoint_on_residual=True, want_misfit=True)
    torch.cuda.synchronize()
    eng.check()
    errs["gradient_ck50"] = rel_l2(ra_ck.cpu().numpy()[0], o_ra)
    parity_report(f"{name} nt={nt} shots={ns}", **errs)
    eng.close()
    assert errs["records"] < REC_TOL
    assert errs["tangent"] < TAN_TOL
    assert errs["gradient"] < GRAD_TOL
    assert errs["misfit"] < MISFIT_TOL
    # checkpointed adjoints recompute the forward segments bitwise
    assert torch.equal(ra_ck, ra) and torch.equal(mf_ck, mf)
