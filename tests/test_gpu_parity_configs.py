"""GPU parity, FP64 form, at the full sizes of the Langevin and batched benchmark
configurations, against the oracle.

* Langevin fluid, 4,194,304 atoms (128 x 128 x 64 FCC cells, rho 0.8442, T 1.0,
  gamma 1, r_c 2.5, skin 0.4, dt 0.005, n_r_df 0, seed 1003): the GPU and the
  oracle draw the same Philox noise, keyed by (seed, id, step), so after 5 steps
  positions and velocities agree within 1e-10 and the temperature within 1e-10
  (the oracle, one core, takes ~7 s per step at this size).
* Kob-Andersen replica, 32,768 atoms (80:20, rho 1.2, T 0.45, gamma 1, dt 0.003,
  per-pair cutoffs 2.5 sigma_ij), run as replica 1 of a two-replica batch: replica
  r draws the noise stream of seed + r, so after 50 steps it equals the oracle's
  single system with seed + 1 within 1e-10.
* The 4096-replica batch (17.5M atoms, NVE): sampled replicas after 20 steps equal
  the oracle's single-system runs within 1e-10.
"""
import numpy as np
import pytest

import cavgpu as G
import workloads as W

pytestmark = pytest.mark.gpu


def wrap_diff(a, b, L):
    d = a - b
    return d - np.round(d / L) * L


def test_langevin_4m_against_oracle(oracle_lib):
    pos, vel, typ, p = W.config_langevin(seed=1003)
    assert len(pos) == 4_194_304
    steps = 5
    s = G.System(pos, vel, typ, p, precision=G.FP64)
    s.setup()
    s.step(steps)
    pg, vg, _ = s.state()
    tg = s.thermo()["temperature"]
    s.close()
    o = oracle_lib.System(pos, vel, typ, p, noise_mode=1)
    o.setup()
    o.step(steps)
    po, vo, _ = o.state()
    to = o.thermo()["temperature"]
    L = p["hi"] - p["lo"]
    assert np.abs(wrap_diff(pg, po, L)).max() <= 1e-10
    assert np.abs(vg - vo).max() <= 1e-10
    assert abs(tg - to) <= 1e-10 * abs(to)


def test_kob_andersen_batch_replica_against_oracle(oracle_lib):
    reps = [W.kob_andersen(n=32768, seed=1005 + r) for r in range(2)]
    p = dict(reps[0][3])
    systems = [(q, v, t, np.asarray(p["lo"], float), np.asarray(p["hi"], float)) for q, v, t, _ in reps]
    b = G.Batch(systems, p, precision=G.FP64)
    b.setup()
    b.step(50)
    pos, vel, _ = b.state()
    pg, vg = b.split(pos)[1], b.split(vel)[1]
    b.close()
    q, v, t, _ = reps[1]
    p1 = dict(p, seed=int(p["seed"]) + 1)
    o = oracle_lib.System(q, v, t, p1, noise_mode=1)
    o.setup()
    o.step(50)
    po, vo, _ = o.state()
    L = np.asarray(p["hi"], float) - np.asarray(p["lo"], float)
    assert np.abs(wrap_diff(pg, po, L)).max() <= 1e-10
    assert np.abs(vg - vo).max() <= 1e-10


def test_replica_batch_4096_sampled_against_oracle(oracle_lib):
    """The 4096-replica benchmark batch itself (17,480,270 atoms, N_r in [256, 8192],
    rho_r in [0.6, 1.0], NVE), FP64, 20 steps: replicas 0, 1, 2047, 4095 and the
    largest one equal the oracle's single-system runs within 1e-10."""
    sets = W.replica_set(4096)
    systems = [(q, v, np.zeros(len(q), np.int32), np.zeros(3), box) for q, v, box, _, _ in sets]
    params = W.lj_params(systems[0][4])
    b = G.Batch(systems, params, precision=G.FP64)
    b.setup()
    b.step(20)
    pos, vel, _ = b.state()
    ps, vs = b.split(pos), b.split(vel)
    b.close()
    largest = int(np.argmax([len(s[0]) for s in systems]))
    for r in sorted({0, 1, 2047, 4095, largest}):
        q, v, t, lo, hi = systems[r]
        p = dict(params, lo=lo, hi=hi)
        o = oracle_lib.System(q, v, t, p, noise_mode=0)
        o.setup()
        o.step(20)
        po, vo, _ = o.state()
        assert np.abs(wrap_diff(ps[r], po, hi - lo)).max() <= 1e-10, r
        assert np.abs(vs[r] - vo).max() <= 1e-10, r
