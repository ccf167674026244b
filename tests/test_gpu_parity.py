"""GPU parity of the MD step (FP64 form) against the reference's fixtures and the oracle.

Bars (from the path's specification):
  * cell assignment and canonical pair set: bit-exact integer sets;
  * forces, virial, kinetic energy, temperature: 1e-12 relative, the per-atom
    force metric being |da_i| / max(|a_i|, rms|a|) so that near-zero net forces
    do not blow it up;
  * NVE trajectories: 1e-10 over 100 steps;
  * Langevin: exact with friction 0; against the oracle's identical Philox
    noise otherwise; temperature statistics for the thermostat.
All GPU calls go through the C ABI (libcavgpu.so via ctypes).
"""
import hashlib

import numpy as np
import pytest

from conftest import golden_cases, golden_params, load_golden, reference_pairs

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-12
TRAJ_ATOL = 1e-10
# cases whose atoms all start inside [lo, hi) (the C ABI rejects others, as
# Atom_data::add_atom(tools::Atom&) does)
CASES = [c for c in golden_cases() if not c.startswith("quirk_")]


@pytest.fixture(scope="module")
def gpu():
    import cavgpu

    return cavgpu


def force_err(a, ref, unit=1.0):
    """max_i |da_i| / max(|a_i|, rms|a|, unit).  `unit` (epsilon/(sigma m) = 1 in reduced
    units) keeps a perfect lattice, whose net forces are rounding residues of ~1e-14,
    from dividing by zero."""
    na = np.linalg.norm(ref, axis=1)
    rms = np.sqrt((na * na).mean()) if len(na) else 1.0
    return float((np.linalg.norm(a - ref, axis=1) / np.maximum(np.maximum(na, rms), unit)).max())


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.fixture(params=CASES)
def case(request, gpu):
    g = load_golden(request.param)
    s = gpu.System(g["pos"], g["vel"], g["typ"], golden_params(g), precision=gpu.FP64)
    s.setup()
    yield request.param, g, s
    s.close()


def virial_terms(g, pairs):
    """Per-pair virial terms -coef*r^2 of the canonical pair rows, with the reference's
    own expression (src/force/lj.cpp:449-489), both orders of every pair."""
    p = golden_params(g)  # the resolved tables of cases with Lj options
    typ = g["typ"]
    L = g["hi"] - g["lo"]
    i, j = pairs[:, 0], pairs[:, 1]
    d = (g["pos"][j] + pairs[:, 2:5] * L) - g["pos"][i]
    r2d = (d * d).sum(1)
    ti, tj = typ[i], typ[j]
    cl = p["cutoff_list"]
    rc = cl[ti, tj] if cl is not None else np.full(len(r2d), float(g["lj_cutoff"]))
    c = rc * rc
    r2 = np.maximum(r2d, p["jump_tol"])  # jump_fix floor (0 when off), after the cutoff test
    eps, sig = p["eps"][ti, tj], p["sigma"][ti, tj]
    rcinv = 1 / c
    rc2 = sig * sig * rcinv
    rc6 = rc2 * rc2 * rc2
    r2i = 1 / r2
    rho2 = sig * sig * r2i
    rho6 = rho2 * rho2 * rho2
    coef = 4 * eps * (-12 * rho6 * rho6 * r2i + 6 * rho6 * r2i + 12 * rc6 * rc6 * rcinv - 6 * rc6 * rcinv)
    keep = (r2d <= c) & (eps != 0)
    if p["ignore_intra_molecule"]:  # pairs inside one molecule take no force (lj.cpp:446)
        keep &= p["molecule_index"][i] != p["molecule_index"][j]
    return (-coef * r2)[keep]


def test_setup_forces(case, oracle_lib):
    import math

    name, g, s = case
    _, _, acc = s.state()
    th = s.thermo()
    assert force_err(acc, g["acc0"]) <= FORCE_RTOL, name
    assert rel(th["ke"], g["ke0"]) <= FORCE_RTOL
    assert rel(th["temperature"], g["t0"]) <= FORCE_RTOL
    # virial: 1e-12 against the exactly summed value; against the reference within the
    # rounding bound of its own sequential sum (n u sum|t|), which dominates on lattices
    o = oracle_lib.System(g["pos"], g["vel"], g["typ"], golden_params(g), noise_mode=0)
    o.setup()
    t = virial_terms(g, o.pairs())
    exact = math.fsum(t) / 2
    scale = np.abs(t).sum() / 2
    assert abs(th["virial"] - exact) <= FORCE_RTOL * max(abs(exact), scale, 1e-300) + 1e-300, name
    bound = (len(t) / 2) * 2.0 ** -53 * scale
    assert abs(th["virial"] - float(g["virial0"])) <= FORCE_RTOL * scale + bound, name


def test_pair_set_bitexact(case):
    name, g, s = case
    pairs = s.pairs()
    if "ignore_intra_molecule" in g:  # the list leaves a molecule's own pairs out
        np.testing.assert_array_equal(pairs, reference_pairs(g))
        assert len(pairs) < int(g["npairs"])
        return
    assert len(pairs) == int(g["npairs"]), name
    if "pairs" in g:
        np.testing.assert_array_equal(pairs, g["pairs"])
    digest = hashlib.sha256(np.ascontiguousarray(pairs, dtype="<i4").tobytes()).hexdigest()
    assert digest == str(g["pairs_sha256"])


def test_outside_start_refused_by_upload(gpu):
    """The reference's quirk_outside_start fixture (an atom placed outside the domain,
    which the reference keeps as another rank's): cavgpu_upload refuses it with
    CAVGPU_E_ARG, as Atom_data::add_atom(tools::Atom &) refuses such an atom
    (src/atom_data/add_unique_atom_molecule.cpp:29-38)."""
    g = load_golden("quirk_outside_start")
    p = golden_params(g)
    outside = ~((g["pos"] >= p["lo"]) & (g["pos"] < p["hi"])).all(1)
    assert outside.sum() == 1
    with pytest.raises(gpu.CavError) as e:
        gpu.System(g["pos"], g["vel"], g["typ"], p, precision=gpu.FP64)
    assert e.value.status == gpu.E_ARG
    inside = ~outside
    s = gpu.System(g["pos"][inside], g["vel"][inside], g["typ"][inside], p, precision=gpu.FP64)
    s.setup()
    s.close()


def test_cells_and_ghosts_bitexact(case):
    name, g, s = case
    if not int(g["use_cell_list"]):
        pytest.skip("reference built no cell list for this case")
    ob, nb = s.bins()
    np.testing.assert_array_equal(nb, g["nbins"])
    np.testing.assert_array_equal(ob, g["bins"])
    src, _, gp, gb = s.ghosts(float(g["ghost_cutoff"]))
    np.testing.assert_array_equal(src, g["ghost_src"])
    np.testing.assert_array_equal(gp, g["ghost_pos"])
    np.testing.assert_array_equal(gb, g["ghost_bins"])


def test_trajectory(case):
    name, g, s = case
    ns = int(g["nsteps"])
    th = s.run(ns, 1)
    pos, vel, acc = s.state()
    L = g["hi"] - g["lo"]
    dp = pos - g["pos_final"]
    dp -= np.round(dp / L) * L  # an atom sitting on a face may be wrapped on one side only
    assert np.abs(dp).max() <= TRAJ_ATOL, name
    assert np.abs(vel - g["vel_final"]).max() <= TRAJ_ATOL, name
    assert force_err(acc, g["acc_final"]) <= 1e-9, name
    # per-step temperature, virial and pressure
    np.testing.assert_allclose(th[:, 1], g["thermo"][:, 0], rtol=1e-9, atol=1e-14)
    if int(g["integrator"]) in (0, 2):  # velocity Verlet, leap-frog: virial of the last force call
        np.testing.assert_allclose(th[:, 3], g["thermo"][:, 1], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(th[:, 2], g["thermo"][:, 2], rtol=1e-9, atol=1e-12)


def test_potential_energy_matches_oracle(gpu, oracle_lib):
    import workloads as W

    pos, vel, typ, p = W.lj_fluid((6, 6, 6), seed=5)
    o = oracle_lib.System(pos, vel, typ, p, noise_mode=0)
    o.setup()
    s = gpu.System(pos, vel, typ, p)
    s.setup()
    vir, pe = s.forces()
    t = o.thermo()
    assert rel(pe, t["pe"]) <= FORCE_RTOL
    assert rel(vir, t["virial"]) <= FORCE_RTOL
    s.close()


def test_thermo_fold_with_many_block_partials(gpu, oracle_lib):
    """500,000 atoms with 32-thread pair-kernel blocks: 15,625 block partials, so each
    thread of the fold's first level (32 blocks x 256) sums two of them and the last
    block folds 32 real sums.  PE and virial against the oracle; the KE recorded at
    every step against the host sum over the downloaded velocities (n_r_df = 3: the
    centre-of-mass part removed).

    The oracle adds the ~13M pair terms of the lattice in one sequential double
    accumulator; the terms of a shell are equal, so its rounding errors share a sign
    and grow as n_pairs * eps (measured 2.3e-10 of the PE): the PE and virial bars
    are that bound.  A partial lost or counted twice by the fold moves the sums by
    ~1/15625 = 6e-5."""
    import workloads as W

    pos, vel, typ, p = W.lj_fluid((50, 50, 50), seed=11)
    o = oracle_lib.System(pos, vel, typ, p, noise_mode=0)
    o.setup()
    t = o.thermo()
    s = gpu.System(pos, vel, typ, p, tpa=1, block=32)
    s.setup()
    vir, pe = s.forces()
    assert rel(pe, t["pe"]) <= 2e-9
    assert rel(vir, t["virial"]) <= 1e-8
    th = s.run(4, 1)
    v = s.state()[1]
    m = p["mass"][typ][:, None]
    mv = (m * v).sum(0)
    ke = 0.5 * ((m * v * v).sum() - float(mv @ mv) / m.sum())
    assert rel(th[-1, 0], ke) <= 1e-12
    s.close()


def test_langevin_noise_matches_oracle(gpu, oracle_lib):
    """Philox noise keyed by (seed, id, step): GPU and oracle draw the same eta."""
    import workloads as W

    pos, vel, typ, p = W.lj_fluid((5, 5, 5), seed=7, integrator=1, friction=1.0, temperature=1.2, n_r_df=0)
    p["seed"] = 12345
    o = oracle_lib.System(pos, vel, typ, p, noise_mode=1)
    o.setup()
    o.step(20)
    s = gpu.System(pos, vel, typ, p)
    s.setup()
    s.step(20)
    po, vo, ao = o.state()
    pg, vg, ag = s.state()
    L = p["hi"] - p["lo"]
    dp = pg - po
    dp -= np.round(dp / L) * L
    assert np.abs(dp).max() < 1e-9
    assert np.abs(vg - vo).max() < 1e-9
    assert rel(s.thermo()["temperature"], o.thermo()["temperature"]) < 1e-9
    s.close()


def test_larger_system_against_oracle(gpu, oracle_lib):
    """16^3 FCC cells (16384 atoms): pair set, cells, forces and 50 NVE steps."""
    import workloads as W

    pos, vel, typ, p = W.lj_fluid((16, 16, 16), seed=99)
    o = oracle_lib.System(pos, vel, typ, p, noise_mode=0)
    o.setup()
    s = gpu.System(pos, vel, typ, p)
    s.setup()
    np.testing.assert_array_equal(s.pairs(), o.pairs())
    ob, nb = s.bins()
    oob, _, onb = o.bins()
    np.testing.assert_array_equal(ob, oob)
    np.testing.assert_array_equal(nb, onb)
    assert force_err(s.state()[2], o.state()[2]) <= FORCE_RTOL
    o.step(50)
    s.step(50)
    po, vo, _ = o.state()
    pg, vg, _ = s.state()
    L = p["hi"] - p["lo"]
    dp = pg - po
    dp -= np.round(dp / L) * L
    assert np.abs(dp).max() <= TRAJ_ATOL
    assert np.abs(vg - vo).max() <= TRAJ_ATOL
    s.close()


@pytest.mark.parametrize("n_r_df", [1, 3])
def test_kinetic_energy_with_fast_centre_of_mass(gpu, oracle_lib, n_r_df):
    """Atom_data::kinetic_energy with n_r_df 1..3 removes the centre-of-mass motion
    (src/atom_data/kinetic_energy.cpp:56-65, the reference subtracting v_cm from each
    atom).  The device folds sum m v^2 and P = sum m v and takes sum m v^2 - |P|^2 / M,
    which cancels when the whole system drifts fast: here every velocity carries a
    uniform offset of 10 x the thermal speed.  KE and T at set-up and after 20 steps
    must still agree with the oracle to 1e-12."""
    import workloads as W

    pos, vel, typ, p = W.lj_fluid((5, 5, 5), seed=17, n_r_df=n_r_df)
    vel = vel + 10.0 * np.sqrt(1.44) * np.array([1.0, -0.6, 0.3])
    p = dict(p, n_r_df=n_r_df)
    s = gpu.System(pos, vel, typ, p, precision=gpu.FP64)
    s.setup()
    o = oracle_lib.System(pos, vel, typ, p, noise_mode=0)
    o.setup()
    for _ in range(2):
        tg, to = s.thermo(), o.thermo()
        assert rel(tg["ke"], to["ke"]) <= FORCE_RTOL, (tg["ke"], to["ke"])
        assert rel(tg["temperature"], to["temperature"]) <= FORCE_RTOL
        s.step(20)
        o.step(20)
    s.close()
