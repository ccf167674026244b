"""Generate the golden fixtures of the MD-step path by running the reference itself.

Builds oracle/_ref/ref_harness (oracle/Makefile target `ref`: the
unmodified caviar-md/caviar-v2 sources compiled as they lie in the reference
checkout, plus a harness that drives their public C++ API), runs it on
seeded synthetic cases and stores inputs + outputs as tests/golden/<case>.npz.

Run from the repository root:   python tests/golden/make_golden.py [REF_DIR]
The GPU machine has no reference checkout; the fixtures travel instead.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, os.path.join(ROOT, "caviar-v2_gb300"))
import workloads as W  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
OUT = os.path.dirname(os.path.abspath(__file__))
FULL_PAIRS_MAX_N = 600


def ext_flags(p):
    """Extension bits of the harness input: jump_tol, WCA, per-atom mixing, lambda tables."""
    return ((1 if p.get("jump_tol") else 0) | (2 if p.get("wca") else 0) | (4 if p.get("eps_atom") is not None else 0)
            | (8 if p.get("lambda_s") is not None else 0) | (16 if p.get("nve") else 0)
            | (32 if p.get("writer") else 0) | (64 if p.get("molecule_index") is not None else 0))


WRITER_KINDS = ("xyz", "energy", "temperature", "pressure", "msd", "volume")
WRITER_FILES = {"xyz": "_xyz.xyz", "energy": "_energy.txt", "temperature": "_temperature.txt",
                "pressure": "_pressure.txt", "msd": "_msd.txt", "volume": "_volume.txt"}


def writer_config(w):
    """int64 [steps of xyz, energy, temperature, pressure, msd, volume; xyz flags; msd_type; msd_initial_step]"""
    flags = (1 if w.get("xyz_id") else 0) | (2 if w.get("xyz_velocity") else 0) | (4 if w.get("xyz_acceleration") else 0)
    return np.array([int(w.get(k, 0)) for k in WRITER_KINDS]
                    + [flags, int(w.get("msd_type", -1)), int(w.get("msd_initial_step", 0))], np.int64)


def write_input(path, pos, vel, typ, p, nsteps):
    nt = int(p["ntypes"])
    cl = p.get("cutoff_list")
    ext = ext_flags(p)
    hdr = np.array([0x48564143, len(pos), nt, nsteps, p["integrator"], p["use_cell_list"], p["n_r_df"],
                    p["pressure_process"], 0 if cl is None else 1, ext], dtype=np.int32)
    dp = np.array(list(p["lo"]) + list(p["hi"]) + [p["nl_cutoff"], p["nl_coef"], p["ghost_cutoff"],
                  p["lj_cutoff"], p["k_b"], p["dt"], p["lang_temperature"], p["lang_friction"],
                  p["lang_kb"]], dtype=np.float64)
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(dp.tobytes())
        f.write(np.asarray(p["eps"], np.float64).reshape(nt, nt).tobytes())
        f.write(np.asarray(p["sigma"], np.float64).reshape(nt, nt).tobytes())
        f.write((np.zeros((nt, nt)) if cl is None else np.asarray(cl, np.float64).reshape(nt, nt)).tobytes())
        f.write(np.asarray(p["mass"], np.float64).tobytes())
        f.write(np.ascontiguousarray(pos, np.float64).tobytes())
        f.write(np.ascontiguousarray(vel, np.float64).tobytes())
        f.write(np.ascontiguousarray(typ, np.int32).tobytes())
        if ext & 1:
            f.write(np.array([p["jump_tol"]], np.float64).tobytes())
        if ext & 4:
            f.write(np.asarray(p["eps_atom"], np.float64).tobytes())
            f.write(np.asarray(p["sigma_atom"], np.float64).tobytes())
        if ext & 8:
            f.write(np.asarray(p["lambda_s"], np.float64).reshape(nt, nt).tobytes())
            f.write(np.asarray(p["lambda_e"], np.float64).reshape(nt, nt).tobytes())
        if ext & 16:
            nve = p["nve"]
            f.write(np.array([nve["step"]], np.int64).tobytes())
            f.write(np.array([nve["mode"], 0], np.int32).tobytes())
            f.write(np.array([nve["value"], nve.get("kb", 0.0)], np.float64).tobytes())
        if ext & 32:
            w = writer_config(p["writer"])
            f.write(w[:6].tobytes())
            f.write(np.array([w[6], w[7], w[8], 0], np.int32).tobytes())
        if ext & 64:
            f.write(np.array([int(bool(p.get("ignore_intra_molecule"))), 0], np.int32).tobytes())
            f.write(np.ascontiguousarray(p["molecule_index"], np.int32).tobytes())


class Reader:
    def __init__(self, buf):
        self.b, self.o = buf, 0

    def take(self, dtype, count):
        a = np.frombuffer(self.b, dtype=dtype, count=count, offset=self.o)
        self.o += a.nbytes
        return a.copy()


def sort_rows(rows):
    if len(rows) == 0:
        return rows.reshape(0, 5)
    order = np.lexsort(tuple(rows[:, k] for k in range(rows.shape[1] - 1, -1, -1)))
    return rows[order]


def pairs_digest(rows):
    return hashlib.sha256(np.ascontiguousarray(rows, dtype="<i4").tobytes()).hexdigest()


def run_case(name, pos, vel, typ, p, nsteps):
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_input(fin, pos, vel, typ, p, nsteps)
        subprocess.run([HARNESS, fin, fout], check=True, stdout=subprocess.DEVNULL)
        r = Reader(open(fout, "rb").read())
        texts = {}
        if p.get("writer"):  # writer::Atom_writer's files, kept byte for byte
            for kind, suffix in WRITER_FILES.items():
                if os.path.exists(fout + suffix):
                    texts["w_" + kind] = np.frombuffer(open(fout + suffix, "rb").read(), np.uint8)
    n, g = r.take(np.int32, 2)
    acc0 = r.take(np.float64, 3 * n).reshape(n, 3)
    virial0, ke0, t0 = r.take(np.float64, 3)
    nb = r.take(np.int32, 3)
    bins = r.take(np.int32, 3 * n).reshape(n, 3)
    gsrc = r.take(np.int32, g)
    gpos = r.take(np.float64, 3 * g).reshape(g, 3)
    gbins = r.take(np.int32, 3 * g).reshape(g, 3)
    (npairs,) = r.take(np.int64, 1)
    pairs = sort_rows(r.take(np.int32, 5 * int(npairs)).reshape(-1, 5))
    (ns,) = r.take(np.int32, 1)
    thermo = r.take(np.float64, 3 * ns).reshape(ns, 3)
    pos_f = r.take(np.float64, 3 * n).reshape(n, 3)
    vel_f = r.take(np.float64, 3 * n).reshape(n, 3)
    acc_f = r.take(np.float64, 3 * n).reshape(n, 3)
    nt = int(p["ntypes"])
    cl = p.get("cutoff_list")
    ext = ext_flags(p)
    extra = {}
    if ext & 14:  # the effective tables after Lj::verify_settings
        extra["eff_eps"] = r.take(np.float64, nt * nt).reshape(nt, nt)
        extra["eff_sigma"] = r.take(np.float64, nt * nt).reshape(nt, nt)
        extra["eff_cutoff_list"] = r.take(np.float64, nt * nt).reshape(nt, nt)
        (extra["eff_cutoff_list_on"],) = r.take(np.int32, 1)
    if ext & 1:
        extra["jump_tol"] = np.float64(p["jump_tol"])
    if ext & 2:
        extra["wca"] = np.int32(1)
    if ext & 4:
        extra["eps_atom"] = np.asarray(p["eps_atom"], np.float64)
        extra["sigma_atom"] = np.asarray(p["sigma_atom"], np.float64)
    if ext & 8:
        extra["lambda_s"] = np.asarray(p["lambda_s"], np.float64).reshape(nt, nt)
        extra["lambda_e"] = np.asarray(p["lambda_e"], np.float64).reshape(nt, nt)
    if ext & 16:
        nve = p["nve"]
        extra["nve"] = np.array([nve["step"], nve["mode"], nve["value"], nve.get("kb", 0.0)], np.float64)
    if ext & 32:
        extra["writer"] = writer_config(p["writer"])
        extra.update(texts)
    if ext & 64:
        extra["molecule_index"] = np.ascontiguousarray(p["molecule_index"], np.int32)
        extra["ignore_intra_molecule"] = np.int32(bool(p.get("ignore_intra_molecule")))
    out = dict(
        # inputs
        pos=pos, vel=vel, typ=typ.astype(np.int32), nsteps=np.int32(nsteps),
        lo=np.asarray(p["lo"]), hi=np.asarray(p["hi"]), ntypes=np.int32(nt),
        nl_cutoff=p["nl_cutoff"], nl_coef=p["nl_coef"], ghost_cutoff=p["ghost_cutoff"], lj_cutoff=p["lj_cutoff"],
        eps=np.asarray(p["eps"]).reshape(nt, nt), sigma=np.asarray(p["sigma"]).reshape(nt, nt),
        cutoff_list=np.zeros((nt, nt)) if cl is None else np.asarray(cl).reshape(nt, nt),
        cutoff_list_on=np.int32(cl is not None), mass=np.asarray(p["mass"]), k_b=p["k_b"], dt=p["dt"],
        integrator=np.int32(p["integrator"]), lang_temperature=p["lang_temperature"],
        lang_friction=p["lang_friction"], lang_kb=p["lang_kb"], n_r_df=np.int32(p["n_r_df"]),
        use_cell_list=np.int32(p["use_cell_list"]), pressure_process=np.int32(p["pressure_process"]),
        # outputs of the reference
        acc0=acc0, virial0=virial0, ke0=ke0, t0=t0, nbins=nb, bins=bins, ghost_src=gsrc, ghost_pos=gpos,
        ghost_bins=gbins, npairs=np.int64(len(pairs)), pairs_sha256=np.array(pairs_digest(pairs)),
        thermo=thermo, pos_final=pos_f, vel_final=vel_f, acc_final=acc_f, **extra,
    )
    if n <= FULL_PAIRS_MAX_N:
        out["pairs"] = pairs
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{name}: N={n} ghosts={g} pairs={len(pairs)} steps={ns} -> {os.path.relpath(path, ROOT)}")


def cases():
    # 256-atom LJ fluid (4^3 FCC cells), cell-list and O(N^2) list builds
    pos, vel, typ, p = W.lj_fluid((4, 4, 4), seed=11)
    yield "fcc256_cell", pos, vel, typ, p, 100
    p2 = dict(p, use_cell_list=0)
    yield "fcc256_brute", pos, vel, typ, p2, 20
    # the N=4000 configuration (10^3 FCC cells, rho 0.8442, T 1.44, rc 2.5, skin 0.3, dt 0.005)
    pos, vel, typ, p = W.config_small_fluid()
    yield "fcc4000_cell", pos, vel, typ, p, 100
    # perturbed lattice with atoms placed exactly on the lower faces and just below the upper faces
    pos, vel, typ, p = W.lj_fluid((5, 5, 5), seed=21)
    rng = np.random.default_rng(22)
    L = p["hi"]
    # move lattice planes next to the faces (x planes just above 0, y and z planes just below L),
    # perturb, then snap coordinates within 0.08 of a face onto it (small moves keep atoms apart)
    pos = np.mod(pos + np.array([-0.40, 0.40, 0.40]) + rng.normal(0.0, 0.03, pos.shape), L)
    for k in np.where(pos[:, 0] < 0.08)[0][:3]:
        pos[k, 0] = 0.0
    for k in np.where(pos[:, 1] > L[1] - 0.08)[0][:3]:
        pos[k, 1] = np.nextafter(L[1], 0.0)
    both = np.where((pos[:, 0] < 0.08) & (pos[:, 2] > L[2] - 0.08))[0][:2]
    pos[both, 0] = 0.0
    pos[both, 2] = np.nextafter(L[2], 0.0)
    yield "perturbed500_cell", pos, vel, typ, p, 40
    # pairs at exactly the list cutoff, inside and across the periodic boundary
    L = 6.0
    p = W.lj_params([L, L, L])
    ce = p["nl_cutoff"] * p["nl_coef"]
    pos = np.array([[0.5, 1.0, 1.0], [0.5 + ce, 1.0, 1.0], [1.0, 3.0, 4.0], [1.0, 3.0 + ce, 4.0],
                    [0.2, 5.0, 2.0], [0.2 + L - ce, 5.0, 2.0], [3.0, 0.3, 5.8], [3.0, 0.3 + L - ce, 5.8],
                    [4.4, 4.4, 0.0], [5.9999999999, 2.2, 2.9]])
    vel = np.zeros_like(pos)
    typ = np.zeros(len(pos), np.int32)
    yield "edge_cutoff_cell", pos, vel, typ, dict(p, n_r_df=0), 10
    # an atom that starts outside the box: Atom_data::set_atoms_mpi_rank marks it foreign once, and
    # kinetic_energy_mpi_domain then leaves it out of KE and T for the whole run
    pos = np.array([[1.0, 1.0, 1.0], [2.2, 1.0, 1.0], [3.0, 4.0, 6.2], [3.0, 4.0, 4.9]])
    yield "quirk_outside_start", pos, np.full_like(pos, 0.1), np.zeros(4, np.int32), dict(p, n_r_df=0), 10
    # Kob-Andersen 80:20, per-pair cutoff list, Langevin with friction 0 (noise term exactly zero)
    pos, vel, typ, p = W.kob_andersen(n=500, seed=31)
    yield "ka500_langevin_nofriction", pos, vel, typ, dict(p, lang_friction=0.0), 50
    # the reference demos' set-up (tests/t001_lj.cpp, tests/t002_lj.cpp), ghost cutoff >= list cutoff
    lo, hi = np.array([-51.0, -50.0, -50.0]), np.array([51.0, 50.0, 50.0])
    p = W.lj_params(hi - lo, rc=5.0, dt=0.001, n_r_df=0, use_cell_list=0)
    p.update(lo=lo, hi=hi, nl_coef=1.0523, ghost_cutoff=5.0 * 1.0523, lj_cutoff=10.0)
    pos = np.array([[-1.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
    yield "t001_two_atoms", pos, np.zeros_like(pos), np.zeros(2, np.int32), p, 200
    g = np.arange(-20, 20, 5, dtype=np.float64)
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    vel = np.random.default_rng(1).uniform(-0.5, 0.5, pos.shape)
    vel -= vel.mean(0)
    yield "t002_grid512", pos, vel, np.zeros(len(pos), np.int32), p, 100
    # leap-frog integrator (Md_simulator::integrate_leap_frog)
    pos, vel, typ, p = W.lj_fluid((5, 5, 5), seed=51, integrator=2)
    yield "fcc500_leapfrog", pos, vel, typ, p, 100
    # Lj jump_fix: r^2 floored at jump_tol inside the cutoff; a few atoms moved close to a neighbour
    pos, vel, typ, p = W.lj_fluid((4, 4, 4), seed=61, temperature=0.5)
    a = (4.0 / 0.8442) ** (1.0 / 3.0)
    for k in range(0, 40, 8):  # atom k+1 is a lattice neighbour of atom k at a / sqrt(2)
        d = pos[k + 1] - pos[k]
        pos[k + 1] = np.mod(pos[k] + d * (0.82 / np.linalg.norm(d)), p["hi"])
    yield "fcc256_jumpfix", pos, vel, typ, dict(p, jump_tol=0.81), 30
    # Lj options resolved in Lj::verify_settings: per-atom Lorentz-Berthelot mixing, WCA cutoffs,
    # lambda scaling of sigma and epsilon (two types, 80:20)
    pos, vel, typ, p = W.kob_andersen(n=864, seed=71, temperature=1.0)
    p = dict(p, integrator=0, lang_friction=0.0, n_r_df=3, cutoff_list=None, wca=1,
             eps_atom=[1.0, 0.6], sigma_atom=[1.0, 0.85],
             lambda_s=[[1.0, 0.95], [0.95, 1.0]], lambda_e=[[1.0, 1.1], [1.1, 0.9]])
    yield "ka864_wca_mixing_lambda", pos, vel, typ, p, 60
    # constraint::Nve velocity rescaling: every 7 steps to k_B T = 1.1 (velocity Verlet), and every
    # step to 1.3 energy per degree of freedom (leap-frog)
    pos, vel, typ, p = W.lj_fluid((5, 5, 5), seed=81)
    yield "fcc500_nve_kbt", pos, vel, typ, dict(p, nve={"step": 7, "mode": 2, "value": 1.1}), 50
    pos, vel, typ, p = W.lj_fluid((4, 4, 4), seed=82, integrator=2)
    yield "fcc256_leapfrog_nve_edof", pos, vel, typ, dict(p, nve={"step": 1, "mode": 0, "value": 1.3}), 40
    # writer::Atom_writer: xyz frames with ids, velocities and accelerations; kinetic energy,
    # temperature, pressure, volume; mean square displacement from step 20 with boundary crossings
    # (lattice planes moved next to the lower x and upper y faces, so that atoms cross them)
    pos, vel, typ, p = W.lj_fluid((4, 4, 4), seed=91)
    pos = np.mod(pos + np.array([-0.41, 0.41, 0.0]), p["hi"])
    wr = {"xyz": 40, "xyz_id": 1, "xyz_velocity": 1, "xyz_acceleration": 1, "energy": 10, "temperature": 10,
          "pressure": 10, "msd": 5, "msd_initial_step": 20, "volume": 30}
    yield "fcc256_writers", pos, vel, typ, dict(p, writer=wr), 100
    # Langevin (friction 0) writer output: the kinetic energy is read after the step, the
    # temperature mid-step; MSD of type 1 only, from step 0
    pos, vel, typ, p = W.kob_andersen(n=500, seed=92, temperature=1.5)
    pos = np.mod(pos + np.array([0.0, 0.0, -0.365]), p["hi"])
    wr = {"xyz": 50, "energy": 5, "temperature": 5, "msd": 10, "msd_type": 1}
    yield "ka500_langevin_writers", pos, vel, typ, dict(p, lang_friction=0.0, writer=wr), 60
    # Lj::ignore_intra_molecule: molecules of four consecutive atoms for the first 400 atoms; the
    # other 100 keep add_atom's molecule index -1 and so count as one molecule among themselves
    pos, vel, typ, p = W.lj_fluid((5, 5, 5), seed=93)
    mol = np.full(len(pos), -1, np.int32)
    mol[:400] = np.arange(400) // 4
    yield "fcc500_ignore_intra", pos, vel, typ, dict(p, ignore_intra_molecule=1, molecule_index=mol), 60
    # constraint::Nve with the Langevin integrator (friction 0): the rescale acts on the
    # mid-step velocities, before the atoms move; every 4 steps to k_B T = 0.6
    pos, vel, typ, p = W.kob_andersen(n=500, seed=94)
    yield "ka500_langevin_nve", pos, vel, typ, dict(p, lang_friction=0.0, nve={"step": 4, "mode": 2, "value": 0.6}), 40


def main():
    # usage: make_golden.py [reference checkout] [case names...]  (no names: every case);
    # the checkout defaults to $CAVIAR2_REF, then to `reference` beside the repository
    default = os.environ.get("CAVIAR2_REF") or os.path.join(os.path.dirname(ROOT), "reference")
    ref = sys.argv[1] if len(sys.argv) > 1 else default
    only = set(sys.argv[2:])
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={ref}", "-j8"], check=True)
    for c in cases():
        if not only or c[0] in only:
            run_case(*c)


if __name__ == "__main__":
    main()
