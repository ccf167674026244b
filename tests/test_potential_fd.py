"""The restated pair potential against the reference's force, by finite differences.

The reference has no potential energy (src/force_field.cpp:39-43 aborts, and
force_field::Lj does not override it); its force on atom i from j is
coef(r) (r_j - r_i) with the shifted coefficient of src/force/lj.cpp:475-484,

    coef = 4 eps (-12 rho^12 / r^2 + 6 rho^6 / r^2 + 12 rho_c^12 / r_c^2 - 6 rho_c^6 / r_c^2),

rho = sigma / r.  The oracle's V(r) (orc_pair_potential, the PE the GPU kernels
reproduce) must be the potential of exactly that force: -dV/dr = -coef(r) r
along r_i - r_j.  This checks it by a fourth-order central difference of V over
r in [0.9 sigma, r_c], for a one-type table and for the Kob-Andersen table with
per-pair cutoffs 2.5 sigma_ij, and checks that V and its slope vanish at r_c.
CPU only.
"""
import numpy as np
import pytest

import workloads as W


def reference_coef(eps, sig, rc, r2):
    """force_field::Lj's forceCoef, in the reference's expression order (src/force/lj.cpp:475-484)."""
    c = rc * rc
    r_c_sq_inv = 1 / c
    rho_c_sq_inv = sig * sig * r_c_sq_inv
    rho_c_6_inv = rho_c_sq_inv * rho_c_sq_inv * rho_c_sq_inv
    rho_c_12_inv = rho_c_6_inv * rho_c_6_inv
    dr_sq_inv = 1 / r2
    rho_sq_inv = sig * sig * dr_sq_inv
    rho_6_inv = rho_sq_inv * rho_sq_inv * rho_sq_inv
    rho_12_inv = rho_6_inv * rho_6_inv
    return 4 * eps * (-12 * rho_12_inv * dr_sq_inv + 6 * rho_6_inv * dr_sq_inv + 12 * rho_c_12_inv * r_c_sq_inv
                      - 6 * rho_c_6_inv * r_c_sq_inv)


def tables():
    one = W.lj_params(np.array([10.0, 10.0, 10.0]))
    _, _, _, ka = W.kob_andersen(n=500, seed=1005)
    return [("one_type", one), ("kob_andersen", ka)]


@pytest.mark.parametrize("name,params", tables(), ids=[t[0] for t in tables()])
def test_force_is_minus_gradient_of_potential(name, params, oracle_lib):
    nt = int(params["ntypes"])
    eps = np.asarray(params["eps"]).reshape(nt, nt)
    sig = np.asarray(params["sigma"]).reshape(nt, nt)
    cl = params.get("cutoff_list")
    V = lambda ti, tj, r: oracle_lib.pair_potential(params, ti, tj, r * r)  # noqa: E731
    worst = 0.0
    for ti in range(nt):
        for tj in range(nt):
            rc = float(np.asarray(cl).reshape(nt, nt)[ti, tj]) if cl is not None else float(params["lj_cutoff"])
            s = float(sig[ti, tj])
            for r in np.linspace(0.9 * s, rc * (1 - 1e-3), 97):
                h = 1e-3 * s
                # fourth-order central difference of V(r)
                dv = (-V(ti, tj, r + 2 * h) + 8 * V(ti, tj, r + h) - 8 * V(ti, tj, r - h) + V(ti, tj, r - 2 * h)) / (12 * h)
                f_ref = -reference_coef(float(eps[ti, tj]), s, rc, r * r) * r  # force on i along r_i - r_j
                scale = max(abs(f_ref), 1e-3 * 24 * float(eps[ti, tj]) / s)
                err = abs(-dv - f_ref) / scale
                worst = max(worst, err)
                assert err < 2e-7, (name, ti, tj, r, -dv, f_ref)
            # continuity at the cutoff: V(rc) = 0 and the one-sided slope tends to 0
            assert abs(V(ti, tj, rc)) < 1e-14 * 4 * float(eps[ti, tj])
            h = 1e-4 * s
            slope = (V(ti, tj, rc) - V(ti, tj, rc - h)) / h
            assert abs(slope) < 1e-3 * 24 * float(eps[ti, tj]) / s
            assert V(ti, tj, rc * 1.001) == 0.0
    assert worst < 2e-7
