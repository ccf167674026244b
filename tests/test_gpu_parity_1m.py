"""GPU parity at the 1,048,576-atom benchmark configuration (FP64 form) against the oracle.

Workload: 64^3 FCC cells x 4 = 1,048,576 atoms, rho 0.8442, T 1.44, r_c 2.5,
skin 0.3, dt 0.005, velocity-Verlet NVE, seed 1002 -- the system the headline
benchmark times.  Bars, as for the small golden cases:
  * canonical pair set (id_i, id_j, image shift) and reference cell assignment
    (Neighborlist::binlist_index, src/neighborlist.cpp:392-414): bit-exact;
  * set-up forces: per-atom |da_i| / max(|a_i|, rms|a|) <= 1e-12;
  * 100 NVE steps: positions (minimum image) and velocities within 1e-10, and the
    cells of the final positions bit-exact.
The oracle (oracle/cav_oracle.c, the reference's serial cell-list path restated)
takes about a minute for the 100 steps.  Pair sets are compared as sorted int64
keys ((i * N + j) * 27 + image code): 79 M rows per side.
"""
import ctypes as C

import numpy as np
import pytest

import workloads as W

pytestmark = pytest.mark.gpu

N_STEPS = 100


def pair_keys(rows, n):
    rows = rows.astype(np.int64)
    code = (rows[:, 2] + 1) + 3 * (rows[:, 3] + 1) + 9 * (rows[:, 4] + 1)
    return np.sort((rows[:, 0] * n + rows[:, 1]) * 27 + code)


def gpu_pair_keys(cavgpu, s):
    lib = cavgpu.lib()
    n = s._check(lib.cavgpu_export_pairs(s._h, None, 0), "export_pairs")
    rows = np.empty((n, 5), np.int32)
    s._check(lib.cavgpu_export_pairs(s._h, C.c_void_p(rows.ctypes.data), n), "export_pairs")
    return pair_keys(rows, s.n)


def oracle_pair_keys(oracle_lib, o):
    lib = oracle_lib.lib()
    n = lib.orc_pair_count(o._h)
    rows = np.empty((n, 5), np.int32)
    got = lib.orc_get_pairs(o._h, rows.ctypes.data_as(C.POINTER(C.c_int32)), n)
    assert got == n
    return pair_keys(rows, o.n)


def force_err(a, ref):
    na = np.linalg.norm(ref, axis=1)
    rms = np.sqrt((na * na).mean())
    return float((np.linalg.norm(a - ref, axis=1) / np.maximum(np.maximum(na, rms), 1.0)).max())


@pytest.fixture(scope="module")
def systems(oracle_lib):
    import cavgpu

    pos, vel, typ, p = W.config_large_fluid(seed=1002)
    assert len(pos) == 1_048_576
    s = cavgpu.System(pos, vel, typ, p, precision=cavgpu.FP64)
    s.setup()
    o = oracle_lib.System(pos, vel, typ, p, noise_mode=0)
    o.setup()
    yield cavgpu, s, o, p
    s.close()


def test_setup_pairs_cells_forces_1m(systems, oracle_lib):
    cavgpu, s, o, p = systems
    ob, nb = s.bins()
    rb, _, rnb = o.bins()
    np.testing.assert_array_equal(nb, rnb)
    np.testing.assert_array_equal(ob, rb)
    kg = gpu_pair_keys(cavgpu, s)
    ko = oracle_pair_keys(oracle_lib, o)
    assert len(kg) == len(ko)
    assert 70 * s.n < len(kg) < 82 * s.n  # ~75.8 list entries per atom
    assert np.array_equal(kg, ko)
    del kg, ko
    _, _, ag = s.state()
    _, _, ao = o.state()
    assert force_err(ag, ao) <= 1e-12
    tg, to = s.thermo(), o.thermo()
    assert abs(tg["ke"] - to["ke"]) <= 1e-12 * abs(to["ke"])
    assert abs(tg["temperature"] - to["temperature"]) <= 1e-12 * abs(to["temperature"])


def test_nve_100_steps_1m(systems):
    cavgpu, s, o, p = systems
    s.step(N_STEPS)
    o.step(N_STEPS)
    pg, vg, ag = s.state()
    po, vo, ao = o.state()
    L = p["hi"] - p["lo"]
    dp = pg - po
    dp -= np.round(dp / L) * L
    assert np.abs(dp).max() <= 1e-10
    assert np.abs(vg - vo).max() <= 1e-10
    assert force_err(ag, ao) <= 1e-9  # the forces follow the positions after 100 steps
    ob, _ = s.bins()
    rb, _, _ = o.bins()
    np.testing.assert_array_equal(ob, rb)
