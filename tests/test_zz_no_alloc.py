"""The allocation-free kinetic-energy entry point against the per-context one.

cavgpu_kinetic_energy_noalloc serves callers that may not allocate device
memory (work recorded into a CUDA graph by stream capture, memory owned by
another allocator, loops that must not synchronise): it takes caller-owned
device arrays and keeps its partial sums in a fixed __device__ array.  Its KE
and T must equal those of cavgpu_thermo after cavgpu_setup on the same
velocities, within the 1e-12 relative tolerance of the other KE/T tests, on two
calls in a row (the second call reuses the scratch the first one left behind),
on a 13,500-atom two-type mixture (7 partial sums) and on the largest system the
scratch serves, 16,777,216 atoms (all 8192 partial sums and the full final fold).

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def system(case):
    import workloads as W

    if case == "ka_13500":  # 2 types, 80:20: 7 partial-sum blocks
        pos, vel, typ, p = W.kob_andersen(n=13500, seed=77)
        return pos, vel, typ, dict(p, mass=np.array([1.0, 2.5]), n_r_df=3, integrator=0)
    # the largest system the scratch array serves: 128 x 128 x 256 FCC cells x 4 =
    # 16,777,216 atoms, every one of the 8192 partial-sum slots in use
    pos, vel, typ, p = W.lj_fluid((128, 128, 256), seed=1002)
    assert len(pos) == 16_777_216
    return pos, vel, typ, p


@pytest.mark.parametrize("case", ["ka_13500", "fluid_16777216"])
def test_noalloc_kinetic_energy_matches_context_thermo(case):
    import torch

    import cavgpu

    pos, vel, typ, p = system(case)
    s = cavgpu.System(pos, vel, typ, p)
    s.setup()
    ref = s.thermo()
    s.close()
    del pos

    dev = torch.device("cuda", 0)
    vel_d = torch.tensor(np.ascontiguousarray(vel), dtype=torch.float64, device=dev)
    typ_d = torch.tensor(typ.astype(np.int64), dtype=torch.int64, device=dev)
    mass = np.ascontiguousarray(p["mass"], dtype=np.float64)
    stream = torch.cuda.current_stream(dev)
    results = []
    for _ in range(2):
        out_d = torch.full((2,), float("nan"), dtype=torch.float64, device=dev)
        rc = cavgpu.lib().cavgpu_kinetic_energy_noalloc(
            len(vel), ctypes.c_void_p(vel_d.data_ptr()), ctypes.c_void_p(typ_d.data_ptr()),
            ctypes.c_void_p(mass.ctypes.data), int(p["ntypes"]), int(p["n_r_df"]), float(p["k_b"]),
            ctypes.c_void_p(out_d.data_ptr()),
            ctypes.c_void_p(stream.cuda_stream))
        assert rc == cavgpu.OK, cavgpu.lib().cavgpu_strerror(rc)
        torch.cuda.synchronize(dev)
        ke, t = out_d.cpu().numpy()
        results.append((ke, t))
        assert abs(ke - ref["ke"]) <= RTOL * abs(ref["ke"]), (ke, ref["ke"])
        assert abs(t - ref["temperature"]) <= RTOL * abs(ref["temperature"]), (t, ref["temperature"])
    assert results[0] == results[1]


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import cavgpu

    one = np.ones(1)
    rc = cavgpu.lib().cavgpu_kinetic_energy_noalloc(16_777_217, ctypes.c_void_p(8), ctypes.c_void_p(8),
                                                    ctypes.c_void_p(one.ctypes.data), 1, 0, 1.0,
                                                    ctypes.c_void_p(8), None)
    assert rc == cavgpu.E_RANGE
