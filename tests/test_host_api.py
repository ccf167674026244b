"""The CAVIAR2-shaped C++ API (caviar-v2_gb300/host/) against the reference's fixtures.

tests/cpp/host_harness.cpp sets each golden case up exactly as a CAVIAR2 user
does (Domain, Atom_data::add_atom(tools::Atom&), Neighborlist, force_field::Lj,
Md_simulator::initialize/setup/step) and writes the reference harness's output
format; the comparison bars are those of tests/test_gpu_parity.py.
"""
import hashlib
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, golden_cases, golden_params, host_harness, load_golden, reference_pairs

sys.path.insert(0, GOLDEN)
import make_golden as MG  # noqa: E402  (input writer / output reader of the harness format)

CASES = [c for c in golden_cases() if not c.startswith("quirk_")]


def harness():
    return host_harness()


def run_host(g, tmp_path, mixed=False):
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    MG.write_input(str(fin), g["pos"], g["vel"], g["typ"], golden_params(g), int(g["nsteps"]))
    cmd = [harness(), str(fin), str(fout)] + (["mixed"] if mixed else [])
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)
    r = MG.Reader(open(fout, "rb").read())
    n, ng = r.take(np.int32, 2)
    out = {"acc0": r.take(np.float64, 3 * n).reshape(n, 3)}
    out["virial0"], out["ke0"], out["t0"] = r.take(np.float64, 3)
    out["nbins"] = r.take(np.int32, 3)
    out["bins"] = r.take(np.int32, 3 * n).reshape(n, 3)
    out["ghost_src"] = r.take(np.int32, ng)
    out["ghost_pos"] = r.take(np.float64, 3 * ng).reshape(ng, 3)
    out["ghost_bins"] = r.take(np.int32, 3 * ng).reshape(ng, 3)
    (npairs,) = r.take(np.int64, 1)
    out["pairs"] = MG.sort_rows(r.take(np.int32, 5 * int(npairs)).reshape(-1, 5))
    (ns,) = r.take(np.int32, 1)
    out["thermo"] = r.take(np.float64, 3 * ns).reshape(ns, 3)
    for k in ("pos_final", "vel_final", "acc_final"):
        out[k] = r.take(np.float64, 3 * n).reshape(n, 3)
    return out


def force_err(a, ref, unit=1.0):
    na = np.linalg.norm(ref, axis=1)
    rms = np.sqrt((na * na).mean())
    return float((np.linalg.norm(a - ref, axis=1) / np.maximum(np.maximum(na, rms), unit)).max())


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_host_api_matches_reference(name, tmp_path):
    g = load_golden(name)
    h = run_host(g, tmp_path)
    assert force_err(h["acc0"], g["acc0"]) <= 1e-12
    assert abs(h["ke0"] - g["ke0"]) <= 1e-12 * abs(g["ke0"])
    assert abs(h["t0"] - g["t0"]) <= 1e-12 * abs(g["t0"])
    if "ignore_intra_molecule" in g:  # the list leaves a molecule's own pairs out
        np.testing.assert_array_equal(h["pairs"], reference_pairs(g))
    else:
        digest = hashlib.sha256(np.ascontiguousarray(h["pairs"], dtype="<i4").tobytes()).hexdigest()
        assert len(h["pairs"]) == int(g["npairs"]) and digest == str(g["pairs_sha256"])
    if int(g["use_cell_list"]):
        np.testing.assert_array_equal(h["nbins"], g["nbins"])
        np.testing.assert_array_equal(h["bins"], g["bins"])
        np.testing.assert_array_equal(h["ghost_src"], g["ghost_src"])
        np.testing.assert_array_equal(h["ghost_pos"], g["ghost_pos"])
        np.testing.assert_array_equal(h["ghost_bins"], g["ghost_bins"])
    L = g["hi"] - g["lo"]
    dp = h["pos_final"] - g["pos_final"]
    dp -= np.round(dp / L) * L
    assert np.abs(dp).max() <= 1e-10
    assert np.abs(h["vel_final"] - g["vel_final"]).max() <= 1e-10
    np.testing.assert_allclose(h["thermo"][:, 0], g["thermo"][:, 0], rtol=1e-9, atol=1e-14)


@pytest.mark.gpu
def test_host_api_mixed_precision_force_error(tmp_path):
    g = load_golden("fcc4000_cell")
    h = run_host(g, tmp_path, mixed=True)
    a, ref = h["acc_final"], g["acc_final"]
    rms = np.sqrt(((a - ref) ** 2).sum(1).mean() / (ref ** 2).sum(1).mean())
    assert rms < 1e-4  # after 100 steps of the mixed form: trajectories drift apart slowly


@pytest.mark.parametrize("name", [c for c in golden_cases() if "eff_eps" in load_golden(c)])
def test_lj_option_tables_match_reference(name, tmp_path):
    """force_field::Lj::verify_settings of the host API (per-atom mixing, WCA, lambda)
    against the tables the reference's own verify_settings produced (CPU only)."""
    g = load_golden(name)
    p = golden_params(g)
    for k in ("jump_tol", "wca", "eps_atom", "sigma_atom", "lambda_s", "lambda_e"):
        if k in g:
            p[k] = g[k]
    # the inputs the reference was given, not the tables it resolved
    p["eps"], p["sigma"] = g["eps"], g["sigma"]
    p["cutoff_list"] = g["cutoff_list"] if int(g["cutoff_list_on"]) else None
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    MG.write_input(str(fin), g["pos"], g["vel"], g["typ"], p, 0)
    subprocess.run([harness(), str(fin), str(fout), "tables"], check=True, stdout=subprocess.DEVNULL)
    r = MG.Reader(open(fout, "rb").read())
    nt = int(g["ntypes"])
    for key in ("eff_eps", "eff_sigma", "eff_cutoff_list"):
        np.testing.assert_array_equal(r.take(np.float64, nt * nt).reshape(nt, nt), g[key])
    assert int(r.take(np.int32, 1)[0]) == int(g["eff_cutoff_list_on"])


def test_host_library_builds_and_loads():
    import ctypes

    harness()
    sys.path.insert(0, os.path.join(ROOT, "caviar-v2_gb300"))
    import build as B

    ctypes.CDLL(B.HOST_LIB)


# (case, status, message, reference site).  Status 1: Log::error_all printed the
# message and exited with 1 (src/log.cpp:193); 2: the setter threw std::runtime_error.
SETTER_ERRORS = [
    ("nl_cutoff", 1, "cutoff have to non-negative.", "src/neighborlist.cpp:206"),
    ("nl_coef", 1, "cutoff_extra_coef must be larger than 1.0", "src/neighborlist.cpp:214"),
    ("lj_cutoff", 2, "Force field cutoff must be non-negative.", "src/force/lj.cpp:77"),
    ("lang_temperature", 1, "Temperature have to non-negative.", "src/md_simulator.cpp:102"),
    ("lang_friction", 1, "friction have to non-negative.", "src/md_simulator.cpp:108"),
    ("integrator", 1, "invalid or non-implemented integrator", "src/md_simulator.cpp:131"),
    ("time_and_step", 1, "cannot use both 'time' and 'step'.", "src/md_simulator.cpp:361"),
    ("no_time_no_step", 1, "please assign 'time' or 'step' variables.", "src/md_simulator.cpp:363"),
    ("nve_kb_alone", 1, "kb and temperature should be set together.", "src/constraint/nve.cpp:109"),
    ("nve_unset", 1, "energy or temperature is not set.", "src/constraint/nve.cpp:116"),
    ("nve_energy_and_kbt", 1, "Only one of 'energy' and 'temperature' can be set.", "src/constraint/nve.cpp:119"),
]


@pytest.mark.parametrize("case,status,message,site", SETTER_ERRORS, ids=[c[0] for c in SETTER_ERRORS])
def test_setter_validation_matches_reference(case, status, message, site):
    """The host API rejects each invalid setting the way the reference does (same
    message; exit through Log::error_all or a thrown std::runtime_error).  CPU only."""
    r = subprocess.run([harness(), "--error", case], capture_output=True, text=True, timeout=60)
    assert r.returncode == status, (site, r.stderr)
    assert message in r.stderr, site


def test_atom_outside_the_domain_is_refused():
    """Deliberate difference: the reference's Atom_data::add_atom(id, type, pos, vel)
    keeps an atom that starts outside the domain and leaves it out of the kinetic
    energy and temperature for the whole run (the quirk_outside_start fixture); the GPU
    path takes atoms inside the domain only, as Atom_data::add_atom(tools::Atom &)
    does (src/atom_data/add_unique_atom_molecule.cpp:29-38).  Md_simulator::initialize
    stops through Log::error_all before any GPU call.  CPU only."""
    r = subprocess.run([harness(), "--error", "outside_start"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1, r.stderr
    assert "the atom with id 1 starts outside the domain" in r.stderr


def test_valid_settings_raise_nothing():
    r = subprocess.run([harness(), "--error", "valid"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "[ERR]" not in r.stderr


@pytest.mark.parametrize("t0,t1,dt", [(0.0, 1.5, 0.5), (2.9, 10.2, 0.003), (0.0, 1.0, 0.005), (3.0, 7.99, 0.01)])
def test_time_mode_steps_match_reference(t0, t1, dt):
    """Md_simulator::set_initial_time/set_final_time: setup() turns the times into
    steps with the reference's expression (int)time / dt (src/md_simulator.cpp:569-573),
    the time truncated before the division: a final time of 1.5 at dt 0.5 gives 2 steps."""
    r = subprocess.run([harness(), "--time-steps", repr(t0), repr(t1), repr(dt)], capture_output=True, text=True,
                       timeout=60, check=True)
    first, last = (int(x) for x in r.stdout.split())
    assert (first, last) == (int(int(t0) / dt), int(int(t1) / dt))


def test_final_add_continues_from_current_step():
    """Md_simulator::set_final_add (src/md_simulator.cpp:92-97): after a run that ended
    at step 100 of 100, 50 more steps run from 100 to 150."""
    r = subprocess.run([harness(), "--final-add", "100", "100", "50"], capture_output=True, text=True, timeout=60,
                       check=True)
    assert r.stdout.split() == ["100", "150"]


@pytest.mark.parametrize("n,nrdf", [(7, 3), (10, 0), (1, 6)])
def test_atom_counts_and_degrees_of_freedom(n, nrdf):
    """Atom_data::get_num_of_atoms_local/global (one rank: both the owned count,
    src/atom_data.cpp:480-497), degree_of_freedoms() = 3N - n_r_df for bondless
    atoms (src/atom_data/kinetic_energy.cpp:642-673) and the process flags."""
    r = subprocess.run([harness(), "--counts", str(n), str(nrdf)], capture_output=True, text=True, timeout=60,
                       check=True)
    assert [int(x) for x in r.stdout.split()] == [n, n, 3 * n - nrdf, 0, 1]


@pytest.mark.parametrize("d", [0.0, 4.9, 5.1, -5.1, 7.0, -7.0, 2.9, 3.1, 12.0])
def test_domain_fix_distance_matches_reference(d):
    """Domain::fix_distance_{x,y,z} (src/domain.cpp:330-398): on a periodic axis one
    shift by the edge when |d| exceeds half of it (12 on a 6-wide axis stays 6);
    non-periodic axes unchanged.  Box 10 x 4 x 6, periodic in x and z."""
    r = subprocess.run([harness(), "--fix-distance", repr(d)], capture_output=True, text=True, timeout=60,
                       check=True)
    x, y, z, vl, vg = (float(v) for v in r.stdout.split())

    def fix(v, edge):
        h = 0.5 * edge
        if v > h:
            v -= h * 2.0
        if v < -h:
            v += h * 2.0
        return v

    assert (x, y, z) == (fix(d, 10.0), d, fix(d, 6.0))
    assert vl == vg == 240.0
