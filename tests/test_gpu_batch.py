"""Batches of independent replicas against the same replicas run one by one.

A batch context (cavgpu_create_batch / cavgpu_upload_batch) advances R periodic
systems of uneven size together: shared pair table and integrator, one box,
cell grid and half-skin rebuild per replica.  Replica r must follow exactly the
trajectory of a single-system context holding only its atoms (Langevin: with
seed + r), because every per-replica list, sum order and noise draw is the
single system's.  The bar is bitwise equality in the FP64 form; the mixed form
is held to the same equality where its arithmetic is per-replica too.
"""
import numpy as np
import pytest

import cavgpu as G
import workloads as W

pytestmark = pytest.mark.gpu


def replicas(n_rep, nmin, nmax, seed):
    # L >= 2 (rc + skin) = 5.6 needs N >= rho * 5.6^3, i.e. N >= 176 at rho 1.0
    return [(pos, vel, np.zeros(len(pos), np.int32), np.zeros(3), box)
            for pos, vel, box, _, _ in W.replica_set(n_rep, nmin, nmax, seed=seed)]


def params_for(systems, **kw):
    return W.lj_params(systems[0][4], **kw)


def run_single(s, params, steps, precision, seed_off=0, **launch):
    p = dict(params)
    p["lo"], p["hi"] = s[3], s[4]
    p["seed"] = int(params["seed"]) + seed_off
    sys_ = G.System(s[0], s[1], s[2], p, precision=precision, **launch)
    sys_.setup()
    if steps:
        sys_.step(steps)
    out = sys_.state(), sys_.thermo(), sys_.stats()
    sys_.close()
    return out


def run_batch(systems, params, steps, precision, **launch):
    b = G.Batch(systems, params, precision=precision, **launch)
    b.setup()
    if steps:
        b.step(steps)
    pos, vel, acc = b.state()
    out = [b.split(pos), b.split(vel), b.split(acc)], b.thermo_batch(), b.stats()
    b.close()
    return out


def wrap_diff(a, b, L):
    d = a - b
    return d - np.round(d / L) * L


@pytest.mark.parametrize("precision", [G.FP64, G.MIXED])
def test_batch_vv_equals_single_runs(precision):
    systems = replicas(24, 180, 1500, seed=2024)
    params = params_for(systems)
    steps = 150
    (bp, bv, ba), bth, bst = run_batch(systems, params, steps, precision)
    assert bst["steps"] == steps
    for r, s in enumerate(systems):
        (p, v, a), th, _ = run_single(s, params, steps, precision)
        if precision == G.FP64:
            np.testing.assert_array_equal(bp[r], p)
            np.testing.assert_array_equal(bv[r], v)
            np.testing.assert_array_equal(ba[r], a)
        else:
            assert np.abs(wrap_diff(bp[r], p, s[4])).max() <= 1e-9
            assert np.abs(bv[r] - v).max() <= 1e-9
        # per-replica thermo: same quantities, folded in another order
        for k, key in enumerate(("ke", "temperature", "pressure", "virial", "pe")):
            assert abs(bth[r, k] - th[key]) <= 1e-11 * max(abs(th[key]), 1.0), (r, key)
        assert bth[r, 5] == pytest.approx(len(s[0]))  # total mass, unit masses


def test_batch_langevin_equals_single_runs_with_replica_seed():
    systems = []
    for k, n in enumerate((256, 500, 864, 256, 500)):
        pos, vel, typ, p = W.kob_andersen(n=n, seed=3000 + k)
        systems.append((pos, vel, typ, np.zeros(3), p["hi"]))
    params = W.kob_andersen(n=256, seed=77)[3]
    steps = 120
    (bp, bv, ba), bth, _ = run_batch(systems, params, steps, G.FP64)
    for r, s in enumerate(systems):
        (p, v, a), th, _ = run_single(s, params, steps, G.FP64, seed_off=r)
        np.testing.assert_array_equal(bp[r], p)
        np.testing.assert_array_equal(bv[r], v)
        np.testing.assert_array_equal(ba[r], a)
        assert abs(bth[r, 1] - th["temperature"]) <= 1e-11 * th["temperature"]


def test_batch_of_one_equals_system():
    pos, vel, typ, params = W.lj_fluid((5, 5, 5), seed=11)
    s = (pos, vel, typ, np.zeros(3), params["hi"])
    (bp, bv, ba), bth, bst = run_batch([s], params, 100, G.FP64)
    (p, v, a), th, st = run_single(s, params, 100, G.FP64)
    np.testing.assert_array_equal(bp[0], p)
    np.testing.assert_array_equal(bv[0], v)
    assert bst["rebuilds"] == st["rebuilds"]
    assert bth[0, 1] == th["temperature"]


def test_batch_rejects_bad_input():
    systems = replicas(3, 200, 300, seed=5)
    params = params_for(systems)
    small = list(systems[1])
    small[4] = np.array([5.0, 8.0, 8.0])  # edge below 2 cutoff_extra
    with pytest.raises(G.CavError):
        G.Batch([systems[0], tuple(small), systems[2]], params)
    b = G.Batch(systems, params)
    b.setup()
    with pytest.raises(G.CavError):
        b.pairs()  # single-system export
    with pytest.raises(G.CavError):
        b.run(10, 5)  # recording is per system
    b.close()
