"""ctypes binding of libcavgpu.so -- the C ABI of include/cavgpu.h.

This is the Python face of the GB300 MD step (used by the tests and by
bench.py); C++ users link the same library through include/cavgpu.h or the
CAVIAR2-shaped host API in caviar-v2_gb300/host/.  There is no fallback: if
libcavgpu.so is missing or no GPU is present, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcavgpu.so")
MAXT = 8

OK, E_ARG, E_CUDA, E_NAN, E_NLIST_OVERFLOW, E_STATE, E_NOMEM, E_RANGE = 0, -1, -2, -3, -4, -5, -6, -7
FP64, MIXED = 0, 1
FORCE_AUTO, FORCE_STRIDED, FORCE_SEGMENTS = 0, 1, 2
NVE_ENERGY_PER_DOF, NVE_ENERGY_TOT, NVE_KBT, NVE_KB_TEMPERATURE = 0, 1, 2, 3
VELOCITY_VERLET, VELOCITY_VERLET_LANGEVIN, LEAP_FROG = 0, 1, 2


class Params(C.Structure):
    """Mirror of struct cavgpu_params (field order and types must match include/cavgpu.h)."""

    _fields_ = [
        ("lo", C.c_double * 3), ("hi", C.c_double * 3), ("bc", C.c_int32 * 3), ("ntypes", C.c_int32),
        ("nl_cutoff", C.c_double), ("nl_coef", C.c_double), ("lj_cutoff", C.c_double),
        ("eps", C.c_double * (MAXT * MAXT)), ("sigma", C.c_double * (MAXT * MAXT)),
        ("cutoff_list", C.c_double * (MAXT * MAXT)), ("cutoff_list_on", C.c_int32), ("integrator", C.c_int32),
        ("mass", C.c_double * MAXT), ("k_b", C.c_double), ("dt", C.c_double), ("lang_temperature", C.c_double),
        ("lang_friction", C.c_double), ("lang_kb", C.c_double), ("lang_kbt", C.c_double), ("seed", C.c_uint64),
        ("n_r_df", C.c_int32), ("pressure_process", C.c_int32), ("precision", C.c_int32), ("noise_off", C.c_int32),
        ("nbr_capacity", C.c_int32), ("threads_per_atom", C.c_int32), ("block_size", C.c_int32),
        ("steps_per_graph", C.c_int32), ("force_kernel", C.c_int32), ("jump_tol", C.c_double),
        ("initial_step", C.c_int64), ("nve_step", C.c_int64), ("nve_mode", C.c_int32), ("nve_pad", C.c_int32),
        ("nve_value", C.c_double), ("nve_kb", C.c_double), ("msd_process", C.c_int32),
        ("ignore_intra_molecule", C.c_int32),
    ]


class CavError(RuntimeError):
    def __init__(self, status, what):
        self.status = status
        extra = ""
        if status == E_CUDA:
            extra = f" [{lib().cavgpu_last_cuda_error().decode()}]"
        super().__init__(f"{what}: {lib().cavgpu_strerror(status).decode()} ({status}){extra}")


# every function include/cavgpu.h declares, with its ctypes signature
_SIGS = {
    "cavgpu_default_params": (None, [C.POINTER(Params)]),
    "cavgpu_create": (C.c_int, [C.POINTER(Params), C.POINTER(C.c_void_p)]),
    "cavgpu_destroy": (None, [C.c_void_p]),
    "cavgpu_upload": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "cavgpu_set_molecules": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cavgpu_setup": (C.c_int, [C.c_void_p]),
    "cavgpu_step": (C.c_int, [C.c_void_p, C.c_int64]),
    "cavgpu_run": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p]),
    "cavgpu_forces": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "cavgpu_thermo": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cavgpu_download": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "cavgpu_download_images": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cavgpu_export_pairs": (C.c_int64, [C.c_void_p, C.c_void_p, C.c_int64]),
    "cavgpu_export_bins": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "cavgpu_export_ghosts": (C.c_int64, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_int64]),
    "cavgpu_stats": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cavgpu_stream": (C.c_void_p, [C.c_void_p]),
    "cavgpu_set_profiling": (C.c_int, [C.c_void_p, C.c_int32]),
    "cavgpu_read_profile": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cavgpu_strerror": (C.c_char_p, [C.c_int]),
    "cavgpu_measure_peaks": (C.c_int, [C.c_void_p]),
    "cavgpu_last_cuda_error": (C.c_char_p, []),
    "cavgpu_kinetic_energy_noalloc": (C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                                C.c_int32, C.c_double, C.c_void_p, C.c_void_p]),
    "cavgpu_create_batch": (C.c_int, [C.POINTER(Params), C.c_int32, C.c_void_p, C.c_void_p,
                                      C.POINTER(C.c_void_p)]),
    "cavgpu_upload_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "cavgpu_thermo_batch": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cavgpu_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
}


def measure_peaks():
    """Measured {fp64, fp32} FMA TFLOP/s of the current device."""
    o = np.zeros(2)
    rc = lib().cavgpu_measure_peaks(_ptr(o))
    if rc:
        raise CavError(rc, "measure_peaks")
    return float(o[0]), float(o[1])

_lib = None


def lib():
    """Load libcavgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def make_params(p, precision=FP64, noise_off=False, tpa=0, block=0, nbr_capacity=0, steps_per_graph=0,
                force_kernel=FORCE_AUTO):
    """cavgpu_params from a parameter dict in the CAVIAR2 setter vocabulary (see workloads.lj_params)."""
    o = Params()
    lib().cavgpu_default_params(C.byref(o))
    nt = int(p["ntypes"])
    for d in range(3):
        o.lo[d], o.hi[d], o.bc[d] = float(p["lo"][d]), float(p["hi"][d]), 1
    o.ntypes = nt
    o.nl_cutoff, o.nl_coef, o.lj_cutoff = float(p["nl_cutoff"]), float(p["nl_coef"]), float(p["lj_cutoff"])
    eps = np.asarray(p["eps"], np.float64).reshape(nt, nt)
    sig = np.asarray(p["sigma"], np.float64).reshape(nt, nt)
    cl = p.get("cutoff_list")
    for a in range(nt):
        for b in range(nt):
            o.eps[a * nt + b], o.sigma[a * nt + b] = eps[a, b], sig[a, b]
            if cl is not None:
                o.cutoff_list[a * nt + b] = np.asarray(cl, np.float64).reshape(nt, nt)[a, b]
    o.cutoff_list_on = int(cl is not None)
    m = np.asarray(p["mass"], np.float64)
    for t in range(nt):
        o.mass[t] = m[t]
    o.k_b, o.dt = float(p["k_b"]), float(p["dt"])
    o.integrator = int(p["integrator"])
    o.lang_temperature, o.lang_friction = float(p["lang_temperature"]), float(p["lang_friction"])
    o.lang_kb, o.lang_kbt = float(p.get("lang_kb", 1.0)), -1.0
    o.seed = int(p.get("seed", 0))
    o.n_r_df, o.pressure_process = int(p["n_r_df"]), int(p.get("pressure_process", 1))
    o.precision, o.noise_off = int(precision), int(bool(noise_off))
    o.threads_per_atom, o.block_size = int(tpa), int(block)
    o.nbr_capacity, o.steps_per_graph = int(nbr_capacity), int(steps_per_graph)
    o.force_kernel = int(force_kernel)
    o.jump_tol = float(p.get("jump_tol", 0.0))
    o.initial_step = int(p.get("initial_step", 0))
    nve = p.get("nve")  # {"step": k, "mode": CAVGPU_NVE_*, "value": x, "kb": y}
    if nve:
        o.nve_step, o.nve_mode = int(nve["step"]), int(nve["mode"])
        o.nve_value, o.nve_kb = float(nve["value"]), float(nve.get("kb", 0.0))
    o.msd_process = int(bool(p.get("msd_process", False)))
    o.ignore_intra_molecule = int(bool(p.get("ignore_intra_molecule", False)))
    return o


class System:
    """One periodic LJ system on the GPU (one cavgpu context)."""

    def __init__(self, pos, vel, typ, params, precision=FP64, noise_off=False, ids=None, **launch):
        self.params = make_params(params, precision, noise_off, **launch)
        h = C.c_void_p()
        rc = lib().cavgpu_create(C.byref(self.params), C.byref(h))
        if rc:
            raise CavError(rc, "cavgpu_create")
        self._h = h
        self.n = len(pos)
        pos = np.ascontiguousarray(pos, np.float64)
        vel = np.ascontiguousarray(vel, np.float64)
        typ = np.ascontiguousarray(typ, np.uint64)
        ids = None if ids is None else np.ascontiguousarray(ids, np.uint64)
        self._check(lib().cavgpu_upload(self._h, self.n, _ptr(pos), _ptr(vel), _ptr(typ), _ptr(ids)), "upload")
        if params.get("molecule_index") is not None:
            mol = np.ascontiguousarray(params["molecule_index"], np.int32)
            self._check(lib().cavgpu_set_molecules(self._h, _ptr(mol)), "set_molecules")

    def _check(self, rc, what):
        if rc < 0:
            raise CavError(rc, what)
        return rc

    def close(self):
        if getattr(self, "_h", None):
            lib().cavgpu_destroy(self._h)
            self._h = None

    __del__ = close

    def setup(self):
        self._check(lib().cavgpu_setup(self._h), "setup")

    def step(self, n=1):
        self._check(lib().cavgpu_step(self._h, n), "step")

    def run(self, n, every):
        out = np.zeros((max(n // every, 1), 5))
        self._check(lib().cavgpu_run(self._h, n, every, _ptr(out)), "run")
        return out[: n // every]

    def forces(self):
        v, pe = C.c_double(), C.c_double()
        self._check(lib().cavgpu_forces(self._h, C.byref(v), C.byref(pe)), "forces")
        return v.value, pe.value

    def thermo(self):
        o = np.zeros(6)
        self._check(lib().cavgpu_thermo(self._h, _ptr(o)), "thermo")
        return dict(ke=o[0], temperature=o[1], pressure=o[2], virial=o[3], pe=o[4], rebuilds=int(o[5]))

    def state(self):
        p, v, a = (np.empty((self.n, 3)) for _ in range(3))
        self._check(lib().cavgpu_download(self._h, _ptr(p), _ptr(v), _ptr(a)), "download")
        return p, v, a

    def images(self):
        """Boundary crossings per atom and axis since the upload (needs msd_process)."""
        m = np.empty((self.n, 3), np.int32)
        self._check(lib().cavgpu_download_images(self._h, _ptr(m)), "download_images")
        return m

    def pairs(self):
        n = self._check(lib().cavgpu_export_pairs(self._h, None, 0), "export_pairs")
        out = np.empty((max(n, 1), 5), np.int32)
        self._check(lib().cavgpu_export_pairs(self._h, _ptr(out), n), "export_pairs")
        return sort_rows(out[:n])

    def bins(self):
        ob, nb = np.empty((self.n, 3), np.int32), np.empty(3, np.int32)
        self._check(lib().cavgpu_export_bins(self._h, _ptr(ob), _ptr(nb)), "export_bins")
        return ob, nb

    def ghosts(self, ghost_cutoff):
        g = self._check(lib().cavgpu_export_ghosts(self._h, ghost_cutoff, None, None, None, None, 0), "ghosts")
        src, sh = np.empty(max(g, 1), np.int32), np.empty((max(g, 1), 3), np.int32)
        gp, gb = np.empty((max(g, 1), 3)), np.empty((max(g, 1), 3), np.int32)
        self._check(lib().cavgpu_export_ghosts(self._h, ghost_cutoff, _ptr(src), _ptr(sh), _ptr(gp), _ptr(gb), g),
                    "ghosts")
        return src[:g], sh[:g], gp[:g], gb[:g]

    def stats(self):
        o = np.zeros(8, np.int64)
        self._check(lib().cavgpu_stats(self._h, _ptr(o)), "stats")
        keys = ("steps", "rebuilds", "max_neighbours", "capacity", "threads_per_atom", "block_size",
                "graph_launches", "kernel_launches")
        return dict(zip(keys, (int(x) for x in o)))

    def stream(self):
        return lib().cavgpu_stream(self._h)

    def autotune(self, trial_steps=0, force=False):
        """Choose the launch shape by timed trials (state restored afterwards)."""
        o = np.zeros(6, np.int64)
        self._check(lib().cavgpu_autotune(self._h, int(trial_steps), int(bool(force)), _ptr(o)), "autotune")
        return dict(threads_per_atom=int(o[0]), block_size=int(o[1]), steps_per_graph=int(o[2]), trials=int(o[3]),
                    force_kernel="segments" if int(o[4]) == FORCE_SEGMENTS else "strided")

    def set_profiling(self, on):
        self._check(lib().cavgpu_set_profiling(self._h, int(on)), "set_profiling")

    def read_profile(self):
        o = np.zeros(2)
        self._check(lib().cavgpu_read_profile(self._h, _ptr(o)), "read_profile")
        return int(o[0]), float(o[1])


class Batch(System):
    """R independent periodic systems advanced together in one context.

    systems: list of (pos, vel, typ, lo3, hi3); all share `params` (pair table,
    integrator, dt, cutoffs).  state() returns the concatenation in that order.
    """

    def __init__(self, systems, params, precision=FP64, noise_off=False, **launch):
        self.params = make_params(params, precision, noise_off, **launch)
        self.nrep = len(systems)
        lo = np.ascontiguousarray([s[3] for s in systems], np.float64)
        hi = np.ascontiguousarray([s[4] for s in systems], np.float64)
        h = C.c_void_p()
        rc = lib().cavgpu_create_batch(C.byref(self.params), self.nrep, _ptr(lo), _ptr(hi), C.byref(h))
        if rc:
            raise CavError(rc, "cavgpu_create_batch")
        self._h = h
        self.counts = np.ascontiguousarray([len(s[0]) for s in systems], np.int64)
        self.n = int(self.counts.sum())
        pos = np.ascontiguousarray(np.concatenate([s[0] for s in systems]), np.float64)
        vel = np.ascontiguousarray(np.concatenate([s[1] for s in systems]), np.float64)
        typ = np.ascontiguousarray(np.concatenate([s[2] for s in systems]), np.uint64)
        self._check(lib().cavgpu_upload_batch(self._h, _ptr(self.counts), _ptr(pos), _ptr(vel), _ptr(typ)),
                    "upload_batch")

    def thermo_batch(self):
        """Per-replica (R, 6) array: KE, T, P, virial, PE, total mass."""
        o = np.zeros((self.nrep, 6))
        self._check(lib().cavgpu_thermo_batch(self._h, _ptr(o)), "thermo_batch")
        return o

    def split(self, a):
        """Split a concatenated per-atom array into the replicas' pieces."""
        return np.split(a, np.cumsum(self.counts)[:-1])


def sort_rows(rows):
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    if len(rows) == 0:
        return rows.reshape(0, 5)
    order = np.lexsort(tuple(rows[:, k] for k in range(rows.shape[1] - 1, -1, -1)))
    return rows[order]
