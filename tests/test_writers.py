"""writer::Atom_writer output: the number text, and the oracle's files against the reference's.

The golden writer cases hold the files the reference's own writer::Atom_writer
wrote (tests/golden/make_golden.py, extension bit 5 of the harness input).  Here
the oracle is stepped on the CPU and its state put through the restated writer
(oracle/writer_text.py): the files must match the reference's byte for byte,
which pins the oracle's boundary-crossing counts, the kinetic energy read after
the step (Langevin: the temperature is taken mid-step) and the MSD conventions.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, golden_cases, golden_params, host_harness, load_golden

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import writer_text as WT  # noqa: E402

WRITER_CASES = [c for c in golden_cases() if "writer" in load_golden(c)]


def golden_texts(g):
    return {k[2:]: g[k].tobytes().decode() for k in g if k.startswith("w_")}


def test_writer_cases_present():
    assert len(WRITER_CASES) >= 2
    for c in WRITER_CASES:
        g = load_golden(c)
        assert {"energy", "temperature", "xyz", "msd"} <= set(golden_texts(g)), c


def test_number_text_matches_ostream():
    """append_general6 (the writers' double-to-text) equals std::ostream's default output."""
    r = subprocess.run([host_harness(), "--format"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout


def test_g6_matches_cpp_examples():
    # values whose text the reference's files hold
    assert WT.g6(0.0) == "0" and WT.g6(-0.0) == "-0" and WT.g6(0.0 + -0.0) == "0"
    assert WT.g6(550.8) == "550.8" and WT.g6(1e-4) == "0.0001" and WT.g6(1e-5) == "1e-05"
    assert WT.g6(1234567.0) == "1.23457e+06" and WT.g6(123456.0) == "123456"


def oracle_files(g, oracle_lib):
    p = golden_params(g)
    s = oracle_lib.System(g["pos"], g["vel"], g["typ"], p, noise_mode=0)
    s.setup()
    w = WT.AtomWriterText(p["writer"], np.asarray(g["hi"]) - np.asarray(g["lo"]))
    typ = np.asarray(g["typ"])

    def emit(i, t, with_pressure):
        th = s.thermo()
        pos, vel, acc = s.state()
        w.write(i, t, th["ke"], th["temperature"], th["pressure"] if with_pressure else 0.0, pos, vel, acc, typ,
                s.images())

    emit(0, 0.0, False)  # Md_simulator::setup: pressure not finalized yet (Atom_data::pressure_ = 0)
    t = 0.0
    for i in range(int(g["nsteps"])):
        s.step(1)
        if w.wants(i):
            emit(i, t, True)
        t += float(g["dt"])
    return w.files()


@pytest.mark.parametrize("case", WRITER_CASES)
def test_oracle_writer_files_match_reference(case, oracle_lib):
    g = load_golden(case)
    ref = golden_texts(g)
    mine = oracle_files(g, oracle_lib)
    assert set(mine) == set(ref), case
    for k in ref:
        assert mine[k] == ref[k], f"{case}: {k} differs from the reference's file"


def test_compare_text_catches_differences():
    a = "0 0 1.5\n10 0.05 2\n"
    assert WT.compare_text(a, a) == 0
    assert WT.compare_text("0 0 1.50001\n10 0.05 2\n", a) == 1
    with pytest.raises(AssertionError):
        WT.compare_text("0 0 1.6\n10 0.05 2\n", a)
    with pytest.raises(AssertionError):
        WT.compare_text("1 0 1.5\n10 0.05 2\n", a)
    with pytest.raises(AssertionError):
        WT.compare_text("0 0 1.5\n", a)
