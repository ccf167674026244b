"""The CPU restatement (oracle/cav_oracle.c) against fixtures produced by the reference itself.

Both sides use the same loop and expression orders and -ffp-contract=off, so
the comparison is bit for bit: forces, virial, kinetic energy, temperature,
cell (bin) assignment, ghost images, the canonical pair set, per-step thermo
and the whole trajectory.
"""
import hashlib

import numpy as np
import pytest

from conftest import golden_cases, golden_params, load_golden

CASES = golden_cases()


@pytest.fixture(params=CASES)
def case(request, oracle_lib):
    g = load_golden(request.param)
    sysm = oracle_lib.System(g["pos"], g["vel"], g["typ"], golden_params(g), noise_mode=0)
    sysm.setup()
    return request.param, g, sysm


def test_setup_forces_bitexact(case):
    name, g, s = case
    _, _, acc = s.state()
    th = s.thermo()
    np.testing.assert_array_equal(acc, g["acc0"], err_msg=name)
    assert th["virial"] == g["virial0"]
    assert th["ke"] == g["ke0"]
    assert th["temperature"] == g["t0"]


def test_ghosts_and_bins_bitexact(case):
    name, g, s = case
    src, _, gpos = s.ghosts()
    np.testing.assert_array_equal(src, g["ghost_src"])
    np.testing.assert_array_equal(gpos, g["ghost_pos"])
    if int(g["use_cell_list"]):
        ob, gb, nb = s.bins()
        np.testing.assert_array_equal(nb, g["nbins"])
        np.testing.assert_array_equal(ob, g["bins"])
        np.testing.assert_array_equal(gb, g["ghost_bins"])


def test_pair_set_bitexact(case):
    name, g, s = case
    pairs = s.pairs()
    assert len(pairs) == int(g["npairs"])
    digest = hashlib.sha256(np.ascontiguousarray(pairs, dtype="<i4").tobytes()).hexdigest()
    assert digest == str(g["pairs_sha256"])
    if "pairs" in g:
        np.testing.assert_array_equal(pairs, g["pairs"])


def test_trajectory_bitexact(case):
    name, g, s = case
    ns = int(g["nsteps"])
    thermo = []
    for _ in range(ns):
        s.step(1)
        t = s.thermo()
        thermo.append([t["temperature"], t["virial"], t["pressure"]])
    pos, vel, acc = s.state()
    np.testing.assert_array_equal(np.array(thermo).reshape(-1, 3), g["thermo"])
    np.testing.assert_array_equal(pos, g["pos_final"])
    np.testing.assert_array_equal(vel, g["vel_final"])
    np.testing.assert_array_equal(acc, g["acc_final"])
