"""Family dispatch + per-family schedules end to end on the GPU, with the result cache."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_family_split_end_to_end(tmp_path):
    import torch
    from seismic_gb300 import schedules as S
    from seismic_gb300 import synthetic
    from seismic_gb300.data import Seismogram, Velocity
    from seismic_gb300.engine import Engine
    from seismic_gb300.geometry import Geometry

    g = Geometry.reference(nt=999)
    rng = np.random.default_rng(11)
    trues = [synthetic.layered(rng), synthetic.faulted(rng)]
    eng = Engine(g, max_models=2)
    tv = torch.as_tensor(np.stack([synthetic.to_vector(v) for v in trues]), device="cuda")
    recs = eng.vel_to_seis(tv)[0]
    samples = []
    for i, v in enumerate(trues):
        start = synthetic.smoothed(v, 4.0)
        seis = Seismogram(data=recs[i].reshape(5, 999, 70).cpu())
        vg = Velocity(data=torch.as_tensor(start), min_vel=torch.tensor(float(v.min()), dtype=torch.float64))
        samples.append(S.Sample(seis, vg, name=f"s{i}", geometry=g))

    def misfit(vel):
        r = eng.vel_to_seis(vel.to_vector().to("cuda").reshape(1, -1))[0][0]
        return float(torch.mean((r - recs_of[id(vel)]) ** 2))

    fs = S.FamilySplit(quick=True, cache_name="split", read_cache=True, write_cache=True)
    runner = S.Runner(cache=S.ResultCache(str(tmp_path)))
    labels = [fs.classify(s) for s in samples]
    assert labels[0] == "FlatVel"                 # laterally flat: mirror-symmetric records
    assert labels[1] in fs.schedules                # synthetic data: whichever family its features pick
    # run the cheap quick chains: the flat model's and the general TV chain for the other
    route = {"s0": "FlatVel", "s1": "TV2D"}
    fs.classify = lambda smp: route[smp.name]
    out = fs.infer(samples, runner)
    assert runner.engine_calls > 0
    for i, (s0, s1) in enumerate(zip(samples, out)):
        recs_of = {id(s0.velocity_guess): recs[i], id(s1.velocity_guess): recs[i]}
        before, after = misfit(s0.velocity_guess), misfit(s1.velocity_guess)
        assert np.isfinite(after) and after < 0.7 * before, (i, before, after)
        assert torch.equal(s1.velocity_guess.data, torch.round(s1.velocity_guess.data))   # both chains round
    # the second call is served from the cache: no engine work, the same models
    calls = runner.engine_calls
    again = fs.infer(samples, runner)
    assert runner.engine_calls == calls
    for a, b in zip(out, again):
        assert torch.equal(a.velocity_guess.data, b.velocity_guess.data)
    runner.close()
    eng.close()
