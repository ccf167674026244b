"""Langevin runs with noise on, checked by statistics (the noise is Philox, not the
reference's unseeded mt19937, so trajectories cannot match the reference).

A 2048-atom LJ fluid with every parameter of the 4,194,304-atom Langevin
benchmark (ρ 0.8442, target T 1.0, γ 1, dt 0.005, r_c 2.5, skin 0.4, n_r_df 0)
is equilibrated and then sampled:
the mean kinetic temperature must sit at the target within the statistical
error (instantaneous T fluctuates by sqrt(2/3N) = 1.8%, ~100 independent
samples in 20,000 steps at a correlation time of ~1/γ = 200 steps, so the mean
is known to ~0.2%; the bound is 1.5%), and the mixed form must reproduce the
FP64 form's mean temperature and radial distribution function.
"""
import numpy as np
import pytest

import cavgpu as G
import workloads as W

pytestmark = pytest.mark.gpu


def rdf(pos, L, rmax=3.0, nbins=60):
    d = pos[:, None, :] - pos[None, :, :]
    d -= np.round(d / L) * L
    r = np.sqrt((d * d).sum(-1))[np.triu_indices(len(pos), 1)]
    h, edges = np.histogram(r, bins=nbins, range=(0.0, rmax))
    shell = 4.0 / 3.0 * np.pi * (edges[1:] ** 3 - edges[:-1] ** 3)
    rho = len(pos) / np.prod(L)
    return h / (shell * rho * len(pos) / 2.0)


def sample(precision):
    pos, vel, typ, params = W.lj_fluid((8, 8, 8), rho=0.8442, temperature=1.0, seed=1003, skin=0.4,
                                       integrator=G.VELOCITY_VERLET_LANGEVIN, friction=1.0, n_r_df=0)
    params["seed"] = 77
    s = G.System(pos, vel, typ, params, precision=precision)
    s.setup()
    s.step(2000)
    temps, g = [], []
    for _ in range(10):
        th = s.run(2000, 20)
        temps.append(th[:, 1])
        p, _, _ = s.state()
        g.append(rdf(p, params["hi"] - params["lo"]))
    s.close()
    return np.concatenate(temps), np.mean(g, axis=0)


def test_langevin_temperature_and_rdf_fp64_vs_mixed():
    t64, g64 = sample(G.FP64)
    tmx, gmx = sample(G.MIXED)
    assert abs(t64.mean() - 1.0) < 0.015, t64.mean()
    assert abs(tmx.mean() - 1.0) < 0.015, tmx.mean()
    assert abs(tmx.mean() - t64.mean()) < 0.015
    # the fluctuations too: instantaneous T spread ~ sqrt(2 / 3N)
    expect = np.sqrt(2.0 / (3 * 2048))
    assert 0.7 * expect < t64.std() < 1.3 * expect
    assert 0.7 * expect < tmx.std() < 1.3 * expect
    # structure: first peak near r = 1.1 and the two RDFs agree bin by bin
    peak = np.argmax(g64) * 0.05 + 0.025
    assert 1.0 < peak < 1.2 and g64.max() > 2.5
    assert np.abs(gmx - g64).max() < 0.15
