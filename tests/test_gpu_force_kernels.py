"""The two pair kernels of the mixed form give the same results bit for bit.

CAVGPU_FORCE_SEGMENTS stages each row segment's neighbourhood in shared memory;
CAVGPU_FORCE_STRIDED gathers neighbours from global memory.  The arithmetic per
pair and the summation order are the same, so forces, velocities and positions
must agree exactly, for velocity Verlet, Langevin and batches of replicas, at
every launch shape.
"""
import numpy as np
import pytest

import cavgpu as G
import workloads as W

pytestmark = pytest.mark.gpu


def run(pos, vel, typ, params, kernel, steps, **launch):
    s = G.System(pos, vel, typ, params, precision=G.MIXED, force_kernel=kernel, **launch)
    s.setup()
    s.step(steps)
    out = s.state(), s.thermo()
    s.close()
    return out


@pytest.mark.parametrize("tpa,block", [(1, 128), (2, 256), (4, 64), (8, 128)])
def test_segment_kernel_equals_strided_vv(tpa, block):
    pos, vel, typ, params = W.lj_fluid((9, 9, 9), seed=31)
    (p1, v1, a1), t1 = run(pos, vel, typ, params, G.FORCE_STRIDED, 120, tpa=tpa, block=block)
    (p2, v2, a2), t2 = run(pos, vel, typ, params, G.FORCE_SEGMENTS, 120, tpa=tpa, block=block)
    np.testing.assert_array_equal(a1, a2)
    np.testing.assert_array_equal(v1, v2)
    np.testing.assert_array_equal(p1, p2)
    assert t1["pe"] == t2["pe"] and t1["virial"] == t2["virial"]


def test_segment_kernel_equals_strided_langevin_two_types():
    pos, vel, typ, params = W.kob_andersen(n=4000, seed=8)
    (p1, v1, _), t1 = run(pos, vel, typ, params, G.FORCE_STRIDED, 80)
    (p2, v2, _), t2 = run(pos, vel, typ, params, G.FORCE_SEGMENTS, 80)
    np.testing.assert_array_equal(v1, v2)
    np.testing.assert_array_equal(p1, p2)


def test_segment_kernel_equals_strided_batch():
    sets = W.replica_set(10, 180, 2000, seed=17)
    systems = [(p, v, np.zeros(len(p), np.int32), np.zeros(3), b) for p, v, b, _, _ in sets]
    params = W.lj_params(systems[0][4])
    res = []
    for kernel in (G.FORCE_STRIDED, G.FORCE_SEGMENTS):
        b = G.Batch(systems, params, precision=G.MIXED, force_kernel=kernel)
        b.setup()
        b.step(60)
        res.append((b.state(), b.thermo_batch()))
        b.close()
    for x, y in zip(res[0][0], res[1][0]):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(res[0][1], res[1][1])


def test_segment_kernel_dense_box():
    # a compressed lattice: cells far fuller than the stage was sized for at set-up
    # density would overflow it only if the density rose; here the box is dense from
    # the start (rho 1.3), exercising large stages and long lists
    pos, vel, typ, params = W.lj_fluid((7, 7, 7), rho=1.3, temperature=0.8, seed=5)
    (p1, v1, _), _ = run(pos, vel, typ, params, G.FORCE_STRIDED, 40)
    (p2, v2, _), _ = run(pos, vel, typ, params, G.FORCE_SEGMENTS, 40)
    np.testing.assert_array_equal(v1, v2)
    np.testing.assert_array_equal(p1, p2)
