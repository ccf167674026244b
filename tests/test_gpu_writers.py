"""writer::Atom_writer on the GPU path against the files the reference wrote.

tests/cpp/host_harness.cpp sets the golden writer cases up through the
CAVIAR2-shaped C++ API (caviar-v2_gb300/host/), steps them on the GPU (FP64) and
lets writer::Atom_writer write its files; they must have the reference's lines and
tokens, integers (steps, types, ids, boundary-crossing totals) identical, and
doubles equal as text or within one unit of the sixth significant digit (the
trajectories agree to ~1e-12, so only values next to a rounding boundary of the
six-digit text can print differently).  The same through Md_simulator::run, which
advances the device in CUDA graphs between the steps the writers read.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, golden_cases, golden_params, host_harness, load_golden

sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import make_golden as MG  # noqa: E402
import writer_text as WT  # noqa: E402

pytestmark = pytest.mark.gpu

WRITER_CASES = [c for c in golden_cases() if "writer" in load_golden(c)]


def harness():
    return host_harness()


def run_writers(g, tmp_path, mode=None):
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    MG.write_input(str(fin), g["pos"], g["vel"], g["typ"], golden_params(g), int(g["nsteps"]))
    subprocess.run([harness(), str(fin), str(fout)] + ([mode] if mode else []), check=True,
                   stdout=subprocess.DEVNULL)
    out = {}
    for kind, suffix in MG.WRITER_FILES.items():
        f = str(fout) + suffix
        if os.path.exists(f):
            out[kind] = open(f).read()
    return out


def check_files(case, mine, g):
    ref = {k[2:]: g[k].tobytes().decode() for k in g if k.startswith("w_")}
    assert set(mine) == set(ref), case
    for k in ref:
        # xyz: accelerations of ~1e-15 (cancelled forces) differ in absolute terms only
        WT.compare_text(mine[k], ref[k], atol=1e-9 if k == "xyz" else 0.0, what=f"{case}:{k}")


@pytest.mark.parametrize("case", WRITER_CASES)
def test_writer_files_step_by_step(case, tmp_path):
    g = load_golden(case)
    check_files(case, run_writers(g, tmp_path), g)


@pytest.mark.parametrize("case", WRITER_CASES)
def test_writer_files_through_run(case, tmp_path):
    g = load_golden(case)
    check_files(case, run_writers(g, tmp_path, "run"), g)


@pytest.mark.parametrize("case", WRITER_CASES)
def test_boundary_crossings_match_oracle(case, oracle_lib):
    import cavgpu

    g = load_golden(case)
    p = dict(golden_params(g), msd_process=True)
    s = cavgpu.System(g["pos"], g["vel"], g["typ"], p, noise_off=True)
    o = oracle_lib.System(g["pos"], g["vel"], g["typ"], p, noise_mode=0)
    s.setup()
    o.setup()
    total = 0
    for k in range(4):
        s.step(25)
        o.step(25)
        np.testing.assert_array_equal(s.images(), o.images(), err_msg=f"{case} after {25 * (k + 1)} steps")
        total = int(np.abs(o.images()).sum())
    assert total > 0 or case.startswith("ka500"), "the case should cross the boundaries"


def test_images_need_msd_process():
    import cavgpu

    g = load_golden(WRITER_CASES[0])
    s = cavgpu.System(g["pos"], g["vel"], g["typ"], dict(golden_params(g), msd_process=False))
    s.setup()
    with pytest.raises(cavgpu.CavError):
        s.images()


def test_langevin_kinetic_energy_after_the_step(oracle_lib):
    """Langevin: KE of the velocities at the end of the step, T from the mid-step velocities."""
    import cavgpu

    g = load_golden("ka500_langevin_writers")
    p = golden_params(g)
    s = cavgpu.System(g["pos"], g["vel"], g["typ"], p, noise_off=True)
    o = oracle_lib.System(g["pos"], g["vel"], g["typ"], p, noise_mode=0)
    s.setup()
    o.setup()
    for n in (1, 7, 30):
        s.step(n)
        o.step(n)
        a, b = s.thermo(), o.thermo()
        assert abs(a["ke"] - b["ke"]) <= 1e-10 * abs(b["ke"])
        assert abs(a["temperature"] - b["temperature"]) <= 1e-10 * abs(b["temperature"])
        _, vel, _ = s.state()
        m = np.asarray(p["mass"])[np.asarray(g["typ"])]
        ke_end = 0.5 * float((m[:, None] * vel * vel).sum())
        assert abs(a["ke"] - ke_end) <= 1e-10 * ke_end


def test_lj_md_driver_outputs(tmp_path):
    """host/lj_md.cpp (the demo-style driver): Md_simulator::run with every writer kind."""
    import json

    harness()
    import build as B

    prefix = str(tmp_path / "o")
    r = subprocess.run([B.LJ_MD, "--cells", "6", "--steps", "300", "--thermo", "20", "--msd", "25", "--xyz", "100",
                        "--no-tune", "--out", prefix], capture_output=True, text=True, check=True)
    rep = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert rep["atoms"] == 864 and rep["steps"] == 300 and rep["atom_steps_per_s"] > 0
    energy = open(prefix + "_energy.txt").read().splitlines()
    # setup's step 0, then steps 0, 20, ..., 280
    assert [int(ln.split()[0]) for ln in energy] == [0] + list(range(0, 300, 20))
    assert [ln.split()[1] for ln in energy[1:3]] == ["0", "0.1"]
    msd = open(prefix + "_msd.txt").read().splitlines()
    assert [int(ln.split()[0]) for ln in msd] == [0, 0] + list(range(25, 300, 25))
    xyz = open(prefix + "_xyz.xyz").read().splitlines()
    assert len(xyz) == 4 * (864 + 2)  # frames at setup and steps 0, 100, 200
    assert xyz[0] == "864" and xyz[1] == "Atom" and len(xyz[2].split()) == 4


def test_time_mode_run_writes_step_times(tmp_path):
    """Md_simulator::set_initial_time / set_final_time through run(): setup() turns
    [1.0, 2.0) at dt 0.005 into steps 200 .. 400 with the reference's (int)time / dt
    (src/md_simulator.cpp:569-573), run() takes exactly those 200 steps, and every row
    the writers emit carries (step i, time i dt) -- setup's own row stays (0, 0), as
    the reference's setup writes it (src/md_simulator.cpp:609-610)."""
    import json

    harness()
    import build as B

    prefix = str(tmp_path / "t")
    r = subprocess.run([B.LJ_MD, "--cells", "4", "--time", "1.0", "2.0", "--thermo", "20", "--no-tune", "--out",
                        prefix], capture_output=True, text=True, check=True)
    rep = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert (rep["initial_step"], rep["final_step"], rep["steps"]) == (200, 400, 200)
    assert rep["current_step"] == 400
    rows = [ln.split() for ln in open(prefix + "_energy.txt").read().splitlines()]
    assert rows[0][:2] == ["0", "0"]
    steps = [int(r[0]) for r in rows[1:]]
    assert steps == list(range(200, 400, 20))
    for r in rows[1:]:
        assert abs(float(r[1]) - int(r[0]) * 0.005) <= 1e-5 * int(r[0]) * 0.005, r

