"""The autotuner (cavgpu_autotune): it must leave the simulation where it found it.

Trials start from a snapshot and the chosen launch shape restarts from it, so
the state after tuning equals the state before, and the trajectory that
follows agrees with an untuned one up to the summation-order rounding of a
different launch shape.
"""
import numpy as np
import pytest

import cavgpu as G
import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [G.FP64, G.MIXED])
def test_autotune_restores_state_and_trajectory(precision):
    pos, vel, typ, params = W.lj_fluid((8, 8, 8), seed=21)
    ref = G.System(pos, vel, typ, params, precision=precision)
    ref.setup()
    ref.step(30)
    s = G.System(pos, vel, typ, params, precision=precision)
    s.setup()
    s.step(30)
    before, st0, th0 = s.state(), s.stats(), s.thermo()
    choice = s.autotune(trial_steps=20, force=True)
    assert choice["threads_per_atom"] in (1, 2, 4, 8) and choice["block_size"] in (64, 128, 256)
    # FP64: 12 shapes + 2 graph lengths; mixed: both pair kernels x 12 shapes + 2
    assert choice["steps_per_graph"] in (25, 50, 100)
    assert choice["trials"] == (14 if precision == G.FP64 else 26)
    assert choice["force_kernel"] in ("segments", "strided")
    after, st1, th1 = s.state(), s.stats(), s.thermo()
    for a, b in zip(before, after):
        np.testing.assert_array_equal(a, b)
    assert st1["steps"] == st0["steps"] and st1["rebuilds"] == st0["rebuilds"]
    assert st1["threads_per_atom"] == choice["threads_per_atom"] and st1["block_size"] == choice["block_size"]
    assert th1["temperature"] == th0["temperature"]
    ref.step(60)
    s.step(60)
    p0, v0, _ = ref.state()
    p1, v1, _ = s.state()
    L = params["hi"] - params["lo"]
    dp = p1 - p0
    dp -= np.round(dp / L) * L
    tol = 1e-9 if precision == G.FP64 else 1e-4
    assert np.abs(dp).max() <= tol and np.abs(v1 - v0).max() <= tol
    # same kind of system: the cached choice, no trials
    again = G.System(pos, vel, typ, params, precision=precision)
    again.setup()
    c2 = again.autotune(trial_steps=20)
    assert c2["trials"] == 0 and c2["threads_per_atom"] == choice["threads_per_atom"]
    for x in (ref, s, again):
        x.close()


def test_autotune_batch_keeps_replicas_independent():
    sets = W.replica_set(12, 180, 900, seed=99)
    systems = [(p, v, np.zeros(len(p), np.int32), np.zeros(3), b) for p, v, b, _, _ in sets]
    params = W.lj_params(systems[0][4])
    b = G.Batch(systems, params, precision=G.FP64)
    b.setup()
    b.step(20)
    th0 = b.thermo_batch()
    b.autotune(trial_steps=10, force=True)
    np.testing.assert_array_equal(b.thermo_batch(), th0)
    b.step(40)
    pos, vel, _ = b.state()
    for r, s in enumerate(systems):
        p = dict(params)
        p["hi"] = s[4]
        one = G.System(s[0], s[1], s[2], p, precision=G.FP64)
        one.setup()
        one.step(60)
        p1, v1, _ = one.state()
        one.close()
        d = b.split(pos)[r] - p1
        d -= np.round(d / s[4]) * s[4]
        assert np.abs(d).max() <= 1e-9 and np.abs(b.split(vel)[r] - v1).max() <= 1e-9
    b.close()
