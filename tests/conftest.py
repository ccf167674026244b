import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
PKG = os.path.join(ROOT, "caviar-v2_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def host_harness():
    """tests/cpp/host_harness.cpp -- a test driver of the CAVIAR2-shaped C++ API --
    compiled against the built libraries into tests/cpp/_build/ (when missing or older
    than its inputs)."""
    import subprocess

    if PKG not in sys.path:
        sys.path.insert(0, PKG)
    import build as B

    if not (os.path.exists(B.LIB) and os.path.exists(B.HOST_LIB)):
        B.build()
    src = os.path.join(ROOT, "tests", "cpp", "host_harness.cpp")
    out_dir = os.path.join(ROOT, "tests", "cpp", "_build")
    exe = os.path.join(out_dir, "host_harness")
    inputs = [src, B.LIB, B.HOST_LIB, os.path.join(PKG, "host", "caviar2_gpu.hpp")]
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(f) for f in inputs):
        os.makedirs(out_dir, exist_ok=True)
        cxx = os.environ.get("CXX", "g++")
        cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", "-I" + os.path.join(ROOT, "include"),
               "-I" + os.path.join(PKG, "host"), src, "-o", exe, "-L" + PKG, "-lcaviar2_gpu", "-lcavgpu",
               "-Wl,-rpath," + PKG]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_cases():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load_golden(name):
    import numpy as np

    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def golden_params(g):
    """Parameter dict (workloads vocabulary) of a golden case."""
    nt = int(g["ntypes"])
    # cases with Lj options carry the tables Lj::verify_settings made of them
    if "eff_eps" in g:
        eps, sigma = g["eff_eps"], g["eff_sigma"]
        cutoff_list = g["eff_cutoff_list"] if int(g["eff_cutoff_list_on"]) else None
    else:
        eps, sigma = g["eps"], g["sigma"]
        cutoff_list = g["cutoff_list"] if int(g["cutoff_list_on"]) else None
    writer = None
    if "writer" in g:  # writer::Atom_writer settings (tests/golden/make_golden.py writer_config)
        w = [int(v) for v in g["writer"]]
        writer = dict(xyz=w[0], energy=w[1], temperature=w[2], pressure=w[3], msd=w[4], volume=w[5],
                      xyz_id=w[6] & 1, xyz_velocity=(w[6] >> 1) & 1, xyz_acceleration=(w[6] >> 2) & 1,
                      msd_type=w[7], msd_initial_step=w[8])
    return dict(
        writer=writer, msd_process=bool(writer and writer["msd"] > 0),
        molecule_index=g["molecule_index"] if "molecule_index" in g else None,
        ignore_intra_molecule=int(g["ignore_intra_molecule"]) if "ignore_intra_molecule" in g else 0,
        lo=g["lo"], hi=g["hi"], ntypes=nt, nl_cutoff=float(g["nl_cutoff"]), nl_coef=float(g["nl_coef"]),
        ghost_cutoff=float(g["ghost_cutoff"]), lj_cutoff=float(g["lj_cutoff"]), eps=eps, sigma=sigma,
        cutoff_list=cutoff_list, jump_tol=float(g["jump_tol"]) if "jump_tol" in g else 0.0,
        nve=None if "nve" not in g else {"step": int(g["nve"][0]), "mode": int(g["nve"][1]),
                                         "value": float(g["nve"][2]), "kb": float(g["nve"][3])},
        mass=g["mass"], k_b=float(g["k_b"]),
        dt=float(g["dt"]), integrator=int(g["integrator"]), lang_temperature=float(g["lang_temperature"]),
        lang_friction=float(g["lang_friction"]), lang_kb=float(g["lang_kb"]), seed=0, n_r_df=int(g["n_r_df"]),
        use_cell_list=int(g["use_cell_list"]), pressure_process=int(g["pressure_process"]),
    )


def reference_pairs(g):
    """The reference's canonical pair set of a golden case as the GPU list holds it:
    with ignore_intra_molecule, pairs inside one molecule are left out of the list
    (the reference keeps them in its list and skips them in the force loop)."""
    rows = g["pairs"]
    if int(g.get("ignore_intra_molecule", 0)):
        mol = g["molecule_index"]
        rows = rows[mol[rows[:, 0]] != mol[rows[:, 1]]]
    return rows


@pytest.fixture(scope="session")
def oracle_lib():
    import cav_oracle

    cav_oracle.build()
    return cav_oracle
