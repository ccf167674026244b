"""ctypes binding of oracle/libcavoracle.so, the CPU restatement of CAVIAR2's MD step.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the GPU library or its host API.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcavoracle.so")
MAXT = 8


class OrcParams(C.Structure):
    _fields_ = [
        ("lo", C.c_double * 3), ("hi", C.c_double * 3), ("bc", C.c_int32 * 3), ("ntypes", C.c_int32),
        ("nl_cutoff", C.c_double), ("nl_coef", C.c_double), ("ghost_cutoff", C.c_double),
        ("lj_cutoff", C.c_double), ("eps", C.c_double * (MAXT * MAXT)), ("sigma", C.c_double * (MAXT * MAXT)),
        ("cutoff_list", C.c_double * (MAXT * MAXT)), ("mass", C.c_double * MAXT), ("k_b", C.c_double),
        ("dt", C.c_double), ("lang_temperature", C.c_double), ("lang_friction", C.c_double),
        ("lang_kb", C.c_double), ("lang_kbt", C.c_double), ("seed", C.c_uint64),
        ("cutoff_list_on", C.c_int32), ("use_cell_list", C.c_int32), ("n_r_df", C.c_int32),
        ("integrator", C.c_int32), ("noise_mode", C.c_int32), ("pressure_process", C.c_int32),
        ("rebuild_test", C.c_int32), ("jump_tol", C.c_double), ("nve_step", C.c_int64), ("nve_mode", C.c_int32),
        ("ignore_intra", C.c_int32), ("nve_value", C.c_double), ("nve_kb", C.c_double),
    ]


def build():
    """Compile libcavoracle.so (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P, D, I32, I64 = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_int64
        L.orc_new.restype = P
        L.orc_new.argtypes = [C.POINTER(OrcParams), C.c_int32, D, D, I32]
        L.orc_free.argtypes = [P]
        L.orc_setup.argtypes = [P]
        L.orc_setup.restype = C.c_int32
        L.orc_step.argtypes = [P, C.c_int32]
        L.orc_step.restype = C.c_int32
        L.orc_get_state.argtypes = [P, D, D, D]
        L.orc_get_thermo.argtypes = [P, D]
        L.orc_get_images.argtypes = [P, I32]
        L.orc_set_molecules.argtypes = [P, I32]
        L.orc_set_molecules.restype = C.c_int32
        L.orc_pair_count.argtypes = [P]
        L.orc_pair_count.restype = I64
        L.orc_get_pairs.argtypes = [P, I32, I64]
        L.orc_get_pairs.restype = I64
        L.orc_ghost_count.argtypes = [P]
        L.orc_ghost_count.restype = C.c_int32
        L.orc_get_ghosts.argtypes = [P, I32, I32, D]
        L.orc_get_bins.argtypes = [P, I32, I32]
        L.orc_get_nbins.argtypes = [P, I32]
        L.orc_pair_potential.argtypes = [C.POINTER(OrcParams), C.c_int32, C.c_int32, C.c_double]
        L.orc_pair_potential.restype = C.c_double
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_langevin_eta.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, D]
        _lib = L
    return _lib


def make_params(p, noise_mode=1):
    """OrcParams from a parameter dict (workloads.lj_params vocabulary)."""
    o = OrcParams()
    nt = int(p["ntypes"])
    for d in range(3):
        o.lo[d] = float(p["lo"][d])
        o.hi[d] = float(p["hi"][d])
        o.bc[d] = 1
    o.ntypes = nt
    o.nl_cutoff, o.nl_coef, o.ghost_cutoff = p["nl_cutoff"], p["nl_coef"], p["ghost_cutoff"]
    o.lj_cutoff = p["lj_cutoff"]
    eps, sig = np.asarray(p["eps"]).reshape(nt, nt), np.asarray(p["sigma"]).reshape(nt, nt)
    cl = p.get("cutoff_list")
    for a in range(nt):
        for b in range(nt):
            o.eps[a * nt + b] = eps[a, b]
            o.sigma[a * nt + b] = sig[a, b]
            if cl is not None:
                o.cutoff_list[a * nt + b] = np.asarray(cl).reshape(nt, nt)[a, b]
    for t in range(nt):
        o.mass[t] = float(np.asarray(p["mass"])[t])
    o.cutoff_list_on = 0 if cl is None else 1
    o.k_b, o.dt = p["k_b"], p["dt"]
    o.lang_temperature, o.lang_friction = p["lang_temperature"], p["lang_friction"]
    o.lang_kb, o.lang_kbt = p.get("lang_kb", 1.0), -1.0
    o.seed = int(p.get("seed", 0))
    o.use_cell_list, o.n_r_df, o.integrator = p["use_cell_list"], p["n_r_df"], p["integrator"]
    o.noise_mode = noise_mode
    o.pressure_process = p.get("pressure_process", 1)
    o.rebuild_test = int(p.get("rebuild_test", 0))
    o.jump_tol = float(p.get("jump_tol", 0.0))
    o.ignore_intra = int(bool(p.get("ignore_intra_molecule", False)))
    nve = p.get("nve")
    if nve:
        o.nve_step, o.nve_mode = int(nve["step"]), int(nve["mode"])
        o.nve_value, o.nve_kb = float(nve["value"]), float(nve.get("kb", 0.0))
    return o


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class System:
    """One oracle system; mirrors Caviar2 + Md_simulator for a single rank."""

    def __init__(self, pos, vel, typ, params, noise_mode=1):
        self.n = len(pos)
        self._p = make_params(params, noise_mode)
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        typ = np.ascontiguousarray(typ, dtype=np.int32)
        self._h = lib().orc_new(C.byref(self._p), self.n, _dp(pos), _dp(vel), _ip(typ))
        if not self._h:
            raise ValueError("orc_new failed")
        if params.get("molecule_index") is not None:
            lib().orc_set_molecules(self._h, _ip(np.ascontiguousarray(params["molecule_index"], np.int32)))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_free(self._h)
            self._h = None

    def setup(self):
        rc = lib().orc_setup(self._h)
        if rc:
            raise RuntimeError(f"orc_setup failed: {rc}")

    def step(self, n=1):
        rc = lib().orc_step(self._h, n)
        if rc:
            raise RuntimeError(f"orc_step failed: {rc}")

    def state(self):
        p, v, a = (np.empty((self.n, 3)) for _ in range(3))
        lib().orc_get_state(self._h, _dp(p), _dp(v), _dp(a))
        return p, v, a

    def images(self):
        """Atom_struct::msd_domain_cross per atom (crossings since construction)."""
        m = np.empty((self.n, 3), np.int32)
        lib().orc_get_images(self._h, _ip(m))
        return m

    def thermo(self):
        o = np.empty(6)
        lib().orc_get_thermo(self._h, _dp(o))
        return dict(ke=o[0], temperature=o[1], pressure=o[2], virial=o[3], pe=o[4], rebuilds=int(o[5]))

    def pairs(self):
        """Canonical (id_i, id_j, sx, sy, sz) rows, sorted lexicographically."""
        n = lib().orc_pair_count(self._h)
        out = np.empty((max(n, 1), 5), dtype=np.int32)
        lib().orc_get_pairs(self._h, _ip(out), n)
        return sort_rows(out[:n])

    def ghosts(self):
        g = lib().orc_ghost_count(self._h)
        src, sh, gp = np.empty(g, np.int32), np.empty((g, 3), np.int32), np.empty((g, 3))
        lib().orc_get_ghosts(self._h, _ip(src), _ip(sh), _dp(gp))
        return src, sh, gp

    def bins(self):
        g = lib().orc_ghost_count(self._h)
        ob, gb, nb = np.empty((self.n, 3), np.int32), np.empty((g, 3), np.int32), np.empty(3, np.int32)
        lib().orc_get_bins(self._h, _ip(ob), _ip(gb))
        lib().orc_get_nbins(self._h, _ip(nb))
        return ob, gb, nb


def sort_rows(rows):
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    if len(rows) == 0:
        return rows.reshape(0, 5)
    order = np.lexsort(tuple(rows[:, k] for k in range(rows.shape[1] - 1, -1, -1)))
    return rows[order]


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in ctr])
    k = (C.c_uint32 * 2)(*[int(x) & 0xFFFFFFFF for x in key])
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return [int(x) for x in o]


def langevin_eta(seed, step, atom_id):
    o = np.empty(3)
    lib().orc_langevin_eta(seed, step, atom_id, _dp(o))
    return o


def pair_potential(params, ti, tj, r2):
    p = make_params(params)
    return lib().orc_pair_potential(C.byref(p), ti, tj, r2)
