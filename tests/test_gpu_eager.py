"""Steps launched from the host (steps_per_graph < 0) equal steps replayed as CUDA graphs.

The eager path launches every rebuild kernel each step (they return at once
unless the half-skin test fired) where the graphs wrap them in conditional
nodes; the work done, and so every result, is the same bit for bit.  Profiling
(CUDA events around each pair-kernel launch) works on both paths.
"""
import numpy as np
import pytest

import cavgpu as G
import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [G.FP64, G.MIXED])
def test_eager_steps_equal_graph_steps(precision):
    pos, vel, typ, params = W.lj_fluid((7, 7, 7), seed=41)
    out = []
    for spg in (0, -1):
        s = G.System(pos, vel, typ, params, precision=precision, steps_per_graph=spg)
        s.setup()
        s.set_profiling(True)
        s.step(75)
        launches, ms = s.read_profile()
        assert launches == 75 and ms > 0.0
        out.append((s.state(), s.thermo(), s.stats()))
        s.close()
    (a, ta, sa), (b, tb, sb) = out
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    assert ta == tb
    assert sa["rebuilds"] == sb["rebuilds"] and sb["graph_launches"] == 0
