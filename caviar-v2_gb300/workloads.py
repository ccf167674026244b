"""Seeded synthetic LJ systems with the shapes of the benchmark configurations.

No public dataset exists for this path; these generators are the whole input.
An FCC lattice (basis {0,0,0},{1/2,1/2,0},{1/2,0,1/2},{0,1/2,1/2}, offset by a
quarter cell) fills a periodic box [0, L); velocities are Gaussian, the
centre-of-mass velocity is removed and they are rescaled so that the
reference's temperature definition (2 KE / (k_B (3N - n_r_df)),
src/atom_data/kinetic_energy.cpp:189-198) equals the target exactly.

Every function returns plain numpy arrays (positions and velocities as
float64 (N, 3), types as int32 (N,)) plus a parameter dict whose keys mirror
the CAVIAR2 setters they stand for.
"""
from __future__ import annotations

import math

import numpy as np

FCC_BASIS = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]])


def fcc_lattice(cells, rho):
    """FCC sites of an (nx, ny, nz)-cell lattice at number density rho.

    Returns (pos (4*nx*ny*nz, 3), box lengths (3,)).  The unit cell edge is
    a = (4/rho)^(1/3) in every direction, so a non-cubic cell count gives an
    orthorhombic box.
    """
    nx, ny, nz = cells
    a = (4.0 / rho) ** (1.0 / 3.0)
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 1, 3)
    pos = (g + FCC_BASIS[None, :, :] + 0.25) * a
    return pos.reshape(-1, 3).astype(np.float64), np.array([nx * a, ny * a, nz * a])


def thermal_velocities(n, temperature, rng, masses=None, n_r_df=3, k_b=1.0):
    """Gaussian velocities, zero net momentum, rescaled to exactly `temperature`."""
    v = rng.normal(0.0, math.sqrt(temperature), size=(n, 3))
    m = np.ones(n) if masses is None else np.asarray(masses, dtype=np.float64)
    v -= (m[:, None] * v).sum(0) / m.sum()
    ke = 0.5 * (m[:, None] * v * v).sum()
    t_now = 2.0 * ke / (k_b * (3 * n - n_r_df))
    return v * math.sqrt(temperature / t_now)


def lj_params(box, ntypes=1, rc=2.5, skin=0.3, dt=0.005, eps=None, sigma=None, cutoff_list=None, mass=None,
              integrator=0, temperature=1.0, friction=0.0, seed=0, n_r_df=3, use_cell_list=1):
    """Parameter dict in the vocabulary of the CAVIAR2 setters."""
    box = np.asarray(box, dtype=np.float64)
    nt = ntypes
    eps = np.ones((nt, nt)) if eps is None else np.asarray(eps, dtype=np.float64)
    sigma = np.ones((nt, nt)) if sigma is None else np.asarray(sigma, dtype=np.float64)
    return dict(
        lo=np.zeros(3), hi=box.copy(), ntypes=nt,
        nl_cutoff=float(rc), nl_coef=float((rc + skin) / rc), ghost_cutoff=float(rc + skin),
        lj_cutoff=float(rc), eps=eps, sigma=sigma,
        cutoff_list=None if cutoff_list is None else np.asarray(cutoff_list, dtype=np.float64),
        mass=np.ones(nt) if mass is None else np.asarray(mass, dtype=np.float64),
        k_b=1.0, dt=float(dt), integrator=int(integrator), lang_temperature=float(temperature),
        lang_friction=float(friction), lang_kb=1.0, seed=int(seed), n_r_df=int(n_r_df),
        use_cell_list=int(use_cell_list), pressure_process=1,
    )


def lj_fluid(cells=(10, 10, 10), rho=0.8442, temperature=1.44, seed=1001, **kw):
    """FCC LJ fluid: N = 4*nx*ny*nz atoms at density rho and temperature T."""
    pos, box = fcc_lattice(cells, rho)
    rng = np.random.default_rng(seed)
    n = len(pos)
    vel = thermal_velocities(n, temperature, rng, n_r_df=kw.get("n_r_df", 3))
    typ = np.zeros(n, dtype=np.int32)
    return pos, vel, typ, lj_params(box, **kw)


def config_small_fluid(seed=1001):
    """N=4000 (10^3 FCC cells), rho 0.8442, T 1.44, rc 2.5, skin 0.3, dt 0.005, NVE."""
    return lj_fluid((10, 10, 10), seed=seed)


def config_large_fluid(seed=1002):
    """N=1,048,576 (64^3 FCC cells), rho 0.8442, T 1.44, rc 2.5, skin 0.3, dt 0.005, NVE."""
    return lj_fluid((64, 64, 64), seed=seed)


def config_langevin(seed=1003, cells=(128, 128, 64)):
    """Langevin LJ: N=4,194,304 on a 128x128x64-cell FCC box (L_x = L_y = 2 L_z),
    rho 0.8442, T 1.0, gamma 1.0, rc 2.5, skin 0.4, dt 0.005."""
    return lj_fluid(cells, rho=0.8442, temperature=1.0, seed=seed, skin=0.4, integrator=1, friction=1.0,
                    n_r_df=0)


def kob_andersen(n=32768, rho=1.2, temperature=0.45, seed=1005, skin=0.3, dt=0.003, friction=1.0):
    """Binary Kob-Andersen 80:20 mixture on an FCC lattice, species by seeded shuffle."""
    cells = round((n / 4) ** (1.0 / 3.0))
    pos, box = fcc_lattice((cells, cells, cells), rho)
    rng = np.random.default_rng(seed)
    n = len(pos)
    typ = np.zeros(n, dtype=np.int32)
    typ[rng.permutation(n)[: int(round(0.2 * n))]] = 1
    vel = thermal_velocities(n, temperature, rng, n_r_df=0)
    eps = np.array([[1.0, 1.5], [1.5, 0.5]])
    sig = np.array([[1.0, 0.8], [0.8, 0.88]])
    cl = 2.5 * sig
    params = lj_params(box, ntypes=2, rc=float(cl.max()), skin=skin, dt=dt, eps=eps, sigma=sig, cutoff_list=cl,
                       integrator=1, temperature=temperature, friction=friction, seed=seed, n_r_df=0)
    return pos, vel, typ, params


def replica_set(n_rep=4096, nmin=256, nmax=8192, rho_range=(0.6, 1.0), t_range=(0.7, 2.0), disp=0.05,
                seed=1004):
    """Independent periodic LJ replicas of uneven size.

    Replica r: N_r ~ U[nmin, nmax], rho_r ~ U[rho_range], T_r ~ U[t_range]; a
    random fill (seeded choice of N_r sites) of a ceil((N_r/4)^(1/3))^3-cell FCC
    lattice spanning the cubic box L = (N_r/rho_r)^(1/3) set by rho_r, plus a
    seeded N(0, disp) displacement.  Returns a list of (pos, vel, box, T_r,
    rho_r) with replica seeds seed + r.
    """
    out = []
    meta_rng = np.random.default_rng(seed)
    ns = meta_rng.integers(nmin, nmax + 1, size=n_rep)
    rhos = meta_rng.uniform(*rho_range, size=n_rep)
    temps = meta_rng.uniform(*t_range, size=n_rep)
    for r in range(n_rep):
        rng = np.random.default_rng(seed + r)
        n = int(ns[r])
        c = math.ceil((n / 4) ** (1.0 / 3.0))
        lat, _ = fcc_lattice((c, c, c), 1.0)
        L = (n / rhos[r]) ** (1.0 / 3.0)
        sites = np.sort(rng.choice(len(lat), size=n, replace=False))
        pos = lat[sites] * (L / (c * (4.0 / 1.0) ** (1.0 / 3.0)))
        pos = np.mod(pos + rng.normal(0.0, disp, size=pos.shape), L)
        pos[pos >= L] = 0.0  # np.mod of a tiny negative number can round up to L
        vel = thermal_velocities(n, float(temps[r]), rng)
        out.append((pos, vel, np.array([L, L, L]), float(temps[r]), float(rhos[r])))
    return out
