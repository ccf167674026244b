"""Langevin statistics at the Kob-Andersen benchmark parameters, FP64 form against mixed.

The batched Kob-Andersen configuration (64 replicas x 32,768 atoms) runs an 80:20
binary mixture at density 1.2 under Langevin dynamics at T 0.45, friction 1,
dt 0.003, with per-pair cutoffs 2.5 sigma_ij (eps_AA 1, eps_AB 1.5, eps_BB 0.5,
sigma_AA 1, sigma_AB 0.8, sigma_BB 0.88).  Its noise is Philox, so trajectories
are compared by their statistics: one 4000-atom replica with exactly those
parameters is equilibrated (5000 steps, 15 time units, ~30 thermostat relaxation
times) and sampled over 20,000 steps.  The mean kinetic temperature must sit at
the target (instantaneous T fluctuates by sqrt(2 / 3N) = 1.3%; ~60 independent
samples put the mean within ~0.2%; the bar is 1%), its spread must match
sqrt(2 / 3N), and the mixed form must reproduce the FP64 form's mean temperature
and its A-A, A-B and B-B radial distribution functions bin by bin.  The
single-type Langevin benchmark's parameters (T 1.0, skin 0.4) are covered the same
way by tests/test_gpu_langevin_stats.py.
"""
import numpy as np
import pytest

import cavgpu as G
import workloads as W

pytestmark = pytest.mark.gpu

N = 4000
T = 0.45


def partial_rdf(pos, typ, L, ta, tb, rmax=3.0, nbins=60):
    a, b = pos[typ == ta], pos[typ == tb]
    d = a[:, None, :] - b[None, :, :]
    d -= np.round(d / L) * L
    r = np.sqrt((d * d).sum(-1))
    if ta == tb:
        r = r[np.triu_indices(len(a), 1)]
        npair = len(a) * (len(a) - 1) / 2
    else:
        r = r.ravel()
        npair = len(a) * len(b)
    h, edges = np.histogram(r, bins=nbins, range=(0.0, rmax))
    shell = 4.0 / 3.0 * np.pi * (edges[1:] ** 3 - edges[:-1] ** 3)
    return h / (shell * npair / np.prod(L))


def sample(precision):
    pos, vel, typ, p = W.kob_andersen(n=N, seed=1005, temperature=T, dt=0.003, friction=1.0)
    assert len(pos) == N and abs((typ == 1).mean() - 0.2) < 1e-3
    p["seed"] = 91
    s = G.System(pos, vel, typ, p, precision=precision)
    s.setup()
    s.step(5000)
    temps, g = [], {k: [] for k in ((0, 0), (0, 1), (1, 1))}
    L = p["hi"] - p["lo"]
    for _ in range(10):
        th = s.run(2000, 20)
        temps.append(th[:, 1])
        x, _, _ = s.state()
        for k in g:
            g[k].append(partial_rdf(x, typ, L, *k))
    s.close()
    return np.concatenate(temps), {k: np.mean(v, axis=0) for k, v in g.items()}


def test_kob_andersen_langevin_temperature_and_rdf_fp64_vs_mixed():
    t64, g64 = sample(G.FP64)
    tmx, gmx = sample(G.MIXED)
    for t in (t64, tmx):
        assert abs(t.mean() - T) < 0.01 * T, t.mean()
        expect = T * np.sqrt(2.0 / (3 * N))
        assert 0.7 * expect < t.std() < 1.3 * expect, t.std()
    assert abs(tmx.mean() - t64.mean()) < 0.01 * T
    # structure: the A-B peak sits near sigma_AB 2^(1/6) ~ 0.9, the A-A peak near 1.1,
    # and the mixed form's partial RDFs follow the FP64 form's
    r = (np.arange(60) + 0.5) * 0.05
    assert 0.75 < r[np.argmax(g64[(0, 1)])] < 1.0
    assert 0.95 < r[np.argmax(g64[(0, 0)])] < 1.2
    for k in g64:
        tol = 0.15 if k != (1, 1) else 0.6  # B-B pairs are few (800 B atoms): noisier
        assert np.abs(gmx[k] - g64[k]).max() < tol, (k, np.abs(gmx[k] - g64[k]).max())
