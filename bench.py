#!/usr/bin/env python3
"""Headline benchmark of the GB300 CAVIAR2 MD step.

Workload (the configuration the metric is quoted on): N = 1,048,576 atoms
(64^3 FCC cells x 4) of LJ fluid, rho 0.8442, T 1.44, r_c 2.5, skin 0.3,
dt 0.005, velocity-Verlet NVE with the list rebuilt on half-skin
displacement.  Seeded synthetic input (no dataset exists for this path).

`value` is the mixed-precision form's atom-steps/s with the state resident
in HBM; the all-FP64 form is timed the same way and reported beside it, with
the ratio.  `e2e` runs the same workload through the C ABI from pinned host
arrays: upload, set-up, K steps with every step's thermo read back, and the
download of the final state all inside the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With torchrun (N > 1) every rank runs its own replica (weak scaling, no
data-path collective); the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "caviar-v2_gb300"))

METRIC = "atom-steps/s, 1M-atom LJ, mixed vs FP64 on 1 GB300 at ≤1e-4 NVE drift"
UNIT = "atom-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=100)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cells", type=int, default=64, help="FCC cells per edge (64 -> 1,048,576 atoms)")
    ap.add_argument("--drift-steps", type=int, default=20000)
    ap.add_argument("--drift-only", action="store_true",
                    help="measure only the NVE energy drift: mixed and FP64 from one equilibrated state, "
                         "--drift-steps steps each, energy sampled every 1000 steps; prints one JSON line")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extra", action="store_true", help="skip the batched and Langevin configurations")
    ap.add_argument("--eager", action="store_true",
                    help="launch every kernel from the host, no CUDA graphs (for profiler runs: profilers "
                         "cannot see the kernels of graphs with conditional nodes); not for timing")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (launch shape from --tpa/--block)")
    ap.add_argument("--tpa", type=int, default=0, help="force-kernel lanes per atom without the autotuner")
    ap.add_argument("--block", type=int, default=0, help="force-kernel block size without the autotuner")
    args = ap.parse_args()
    if args.eager:
        LAUNCH["steps_per_graph"] = -1
    if args.tpa:
        LAUNCH["tpa"] = args.tpa
    if args.block:
        LAUNCH["block"] = args.block
    return args


# launch options given to every context (--eager: steps_per_graph = -1)
LAUNCH = {}


# ---------------------------------------------------------------------------
def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=ws)
    return ws, rank, local


def relaunch_under_torchrun(argv, n):
    """`--gpus N` (N > 1) without a launcher: start N ranks of this script through
    torch.distributed.run on this node (127.0.0.1) and return their exit status."""
    port = 29500 + os.getpid() % 2000
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(n),
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + list(argv)
    return subprocess.call(cmd)


def replica_share(n_rep, ws, rank):
    """Replicas of a batch that rank `rank` of `ws` runs: r = rank, rank + ws, ...
    (round robin: every rank's share holds the same spread of sizes).  The replicas
    are independent systems, so the shares need no communication."""
    return list(range(rank, n_rep, ws))


def sum_over_ranks(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock / throttle-reason samples every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev_id):
        self.dev_id = dev_id
        self.proc = None

    def __enter__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        cmd = ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200"]
        if self.dev_id:
            cmd += ["-i", self.dev_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            self.proc.wait()
        self.f.flush()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines()]
            os.unlink(self.f.name)
        except OSError:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm, smax, reasons = [], [], set()
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def gpu_uuid():
    try:
        import torch

        u = str(torch.cuda.get_device_properties(0).uuid)
        return u if u.startswith("GPU-") else "GPU-" + u
    except Exception:
        return None


# ---------------------------------------------------------------------------
def cpu_reference_rate(pos, vel, typ, params, steps, warmup):
    """The reference's CPU path (oracle/cav_oracle.c, a restatement of the reference's
    single-rank serial loop: ghost exchange, cell list, Verlet list, LJ, VV) on a
    bounded sample: set-up untimed, `warmup` steps untimed, `steps` steps timed."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import cav_oracle

    cav_oracle.build()
    s = cav_oracle.System(pos, vel, typ, params, noise_mode=0)
    s.setup()
    if warmup:
        s.step(warmup)
    t0 = time.perf_counter()
    s.step(steps)
    dt = time.perf_counter() - t0
    return len(pos) * steps / dt, dt


def fused_fraction(steps, tuned, spg_default=50):
    """Share of the timed pair-kernel launches that also drift the next step: in
    each chunk of S steps (one CUDA graph) every step but the last drifts the next,
    made even in number (cav_api.cu, make_plan), velocity Verlet without records."""
    spg = (tuned or {}).get("steps_per_graph") or spg_default
    spg = LAUNCH.get("steps_per_graph", spg)
    if spg <= 0:
        spg = spg_default
    fused, left = 0, steps
    while left > 0:
        sz = min(left, spg)
        fused += (sz - 1) - ((sz - 1) % 2)
        left -= sz
    return fused / max(steps, 1)


def cpu_model():
    """The host CPU's model name (lscpu), for the CPU baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform

    return platform.machine()


def read_profile_traffic(name):
    """dram bytes per launch recorded in a committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.strip().startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        return {}


def time_device(cavgpu, torch, pos, vel, typ, params, precision, steps, warmup, ws, sampler_id, tune=True):
    """Device-resident timing: events on the context's stream around K steps
    (launch shape chosen by cavgpu_autotune first, outside the timed region)."""
    s = cavgpu.System(pos, vel, typ, params, precision=precision, **LAUNCH)
    s.setup()
    choice = s.autotune(trial_steps=30) if tune else None
    s.step(warmup)
    stream = torch.cuda.ExternalStream(s.stream())
    # one untimed call of the timed call's shape: its CUDA graphs (cached per chunk
    # size, record period and profiling) are captured and instantiated here, not in
    # the timed region, where that host work would leave the GPU idle
    s.set_profiling(True)
    s.step(steps)
    s.set_profiling(True)  # the launch times counted from here
    st0 = s.stats()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    barrier(ws)
    with ClockSampler(sampler_id) as cs:
        e0.record(stream)
        s.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    ms = e0.elapsed_time(e1)
    st1 = s.stats()
    nlaunch, force_ms = s.read_profile()
    s.set_profiling(False)
    nbar = s._check(cavgpu.lib().cavgpu_export_pairs(s._h, None, 0), "pairs") / len(pos)
    out = dict(ms=ms, force_ms=force_ms, force_launches=nlaunch, rebuilds=st1["rebuilds"] - st0["rebuilds"],
               kernel_launches=st1["kernel_launches"] - st0["kernel_launches"], nbar=nbar,
               clocks=cs.summary(), tpa=st1["threads_per_atom"], block=st1["block_size"],
               capacity=st1["capacity"], autotune=choice)
    return s, out


def time_batch(cavgpu, torch, systems, params, precision, steps, warmup, trial_steps, ws=1):
    """A batch of replicas, device-resident: autotune, warm-up, K timed steps.  With
    ws > 1 ranks, each runs its own share of the replicas; the timed region is
    bracketed by barriers and its time is the max over ranks.  Returns throughput
    over all replicas of all ranks and this rank's per-replica thermo after the run."""
    b = cavgpu.Batch(systems, params, precision=precision, **LAUNCH)
    b.setup()
    choice = b.autotune(trial_steps=trial_steps)
    b.step(warmup)
    stream = torch.cuda.ExternalStream(b.stream())
    b.set_profiling(True)
    b.step(steps)  # the timed call's graphs captured outside the timed region
    b.set_profiling(True)
    st0 = b.stats()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    barrier(ws)
    e0.record(stream)
    b.step(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    ms = max_over_ranks(ws, e0.elapsed_time(e1))
    atoms = sum_over_ranks(ws, b.n)
    reps = sum_over_ranks(ws, b.nrep)
    st1 = b.stats()
    nl, fms = b.read_profile()
    th = b.thermo_batch()
    out = dict(value=atoms * steps / (ms * 1e-3), ms_per_step=ms / steps, steps=steps, warmup=warmup,
               atoms=int(atoms), replicas=int(reps), ranks=ws, force_ms_per_launch=fms / max(nl, 1),
               replica_rebuilds=st1["rebuilds"] - st0["rebuilds"],
               gpu_launches=st1["kernel_launches"] - st0["kernel_launches"], autotune=choice)
    b.close()
    return out, th


def extra_workloads(cavgpu, torch, W, np, single_mixed, ws=1, rank=0):
    """The other benchmark configurations, each timed on this GPU beside the headline:
    4096 uneven replicas (mixed and FP64), 64 Kob-Andersen replicas (mixed Langevin),
    split over the ranks (replica_share), then -- on rank 0 -- the 4,194,304-atom
    Langevin fluid (mixed and FP64) and the writer runs."""
    res = {}
    sets = W.replica_set(4096)
    mine = replica_share(len(sets), ws, rank)
    systems = [(p, v, np.zeros(len(p), np.int32), np.zeros(3), b) for p, v, b, _, _ in (sets[r] for r in mine)]
    params = W.lj_params(systems[0][4])
    m, _ = time_batch(cavgpu, torch, systems, params, cavgpu.MIXED, 200, 20, 10, ws)
    f, _ = time_batch(cavgpu, torch, systems, params, cavgpu.FP64, 20, 3, 4, ws)
    res["replicas_4096"] = {
        "workload": "4096 periodic LJ replicas, N_r ~ U[256, 8192], rho_r ~ U[0.6, 1.0], T_r ~ U[0.7, 2.0], "
                    "random FCC fill + N(0, 0.05) displacement, rc 2.5, skin 0.3, dt 0.005, NVE",
        "mixed": m, "fp64": f, "mixed_over_single_system_mixed": m["value"] / ws / single_mixed}
    del systems, sets
    systems = []
    for r in replica_share(64, ws, rank):
        pos, vel, typ, p = W.kob_andersen(n=32768, seed=1005 + r)
        systems.append((pos, vel, typ, np.zeros(3), p["hi"]))
    params = W.kob_andersen(n=32768, seed=1005)[3]
    k, th = time_batch(cavgpu, torch, systems, params, cavgpu.MIXED, 400, 20, 20, ws)
    k["mean_T_over_replicas"] = sum_over_ranks(ws, float(th[:, 1].sum())) / 64
    res["kob_andersen_64x32768"] = {
        "workload": "64 replicas x 32768 atoms, Kob-Andersen 80:20, rho 1.2, Langevin T 0.45 gamma 1, dt 0.003",
        "mixed": k}
    del systems
    if rank != 0:
        return res
    pos, vel, typ, params = W.config_langevin()
    lang = {"workload": "Langevin LJ fluid, 4,194,304 atoms (128x128x64 FCC cells), T 1.0, gamma 1, skin 0.4"}
    for prec, name, steps in ((cavgpu.MIXED, "mixed", 400), (cavgpu.FP64, "fp64", 40)):
        s = cavgpu.System(pos, vel, typ, params, precision=prec, **LAUNCH)
        s.setup()
        s.autotune(trial_steps=10)
        s.step(10)
        s.step(steps)  # the timed call's graphs captured outside the timed region
        stream = torch.cuda.ExternalStream(s.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        s.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        lang[name] = {"value": len(pos) * steps / (ms * 1e-3), "ms_per_step": ms / steps, "steps": steps,
                      "T_end": s.thermo()["temperature"]}
        s.close()
    res["langevin_4M"] = lang
    res["writers_1M"] = writer_runs()
    return res


def writer_runs(steps=2000):
    """Md_simulator::run through the C++ API (host/lj_md.cpp) on the 1,048,576-atom fluid
    (mixed), without writers and with writer::Atom_writer output: kinetic energy,
    temperature and pressure every 100 steps, MSD every 100, xyz frames every 1000."""
    import json
    import subprocess
    import tempfile

    import build as B

    out = {"workload": "LJ fluid 1,048,576 atoms (64^3 FCC cells), mixed, velocity Verlet, "
                       f"{steps} steps through Md_simulator::run; wall time of run()"}
    with tempfile.TemporaryDirectory() as td:
        for name, extra in (("no_writers", []), ("writers", ["--thermo", "100", "--msd", "100", "--xyz", "1000"])):
            cmd = [B.LJ_MD, "--cells", "64", "--steps", str(steps), "--mixed", "--out", os.path.join(td, "o")] + extra
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                out[name] = {"error": (r.stderr or r.stdout).strip()[-300:]}
                continue
            out[name] = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
        if "run_s" in out.get("writers", {}) and "run_s" in out.get("no_writers", {}):
            out["writers_over_no_writers"] = out["writers"]["atom_steps_per_s"] / out["no_writers"]["atom_steps_per_s"]
            out["xyz_bytes_per_frame"] = os.path.getsize(os.path.join(td, "o_xyz.xyz")) // 3
    return out


def nve_drift(cavgpu, pos, vel, typ, params, precision, steps, every=100, series=False):
    """NVE energy drift: least-squares slope of E = KE + PE sampled every `every`
    steps over `steps` steps, per 1e6 steps and relative to the mean |E|; and the
    largest |E - E_first| / |E| seen (with series, also the sampled E).  None when
    steps is 0."""
    import numpy as np

    if steps <= 0:
        return (None, None, None) if series else (None, None)
    s = cavgpu.System(pos, vel, typ, params, precision=precision, **LAUNCH)
    s.setup()
    th = s.run(steps, every)
    s.close()
    e = th[:, 0] + th[:, 4]
    t = (1 + np.arange(len(e))) * every
    slope = np.polyfit(t, e, 1)[0]
    out = (float(slope * 1e6 / abs(e.mean())), float(np.abs(e - e[0]).max() / abs(e.mean())))
    return out + (e,) if series else out


def drift_only(args, cavgpu, W, np):
    """The NVE energy drift of the 1,048,576-atom fluid over --drift-steps steps, mixed
    and FP64 from one state (the lattice melted by 5000 mixed steps), E = KE + PE
    sampled every 1000 steps.  One JSON line."""
    pos, vel, typ, params = W.lj_fluid((args.cells,) * 3, seed=1002)
    eq = cavgpu.System(pos, vel, typ, params, precision=cavgpu.MIXED, **LAUNCH)
    eq.setup()
    eq.step(5000)
    p_eq, v_eq, _ = eq.state()
    eq.close()
    out = {"workload": f"lj_fluid_{len(pos)}_atoms_nve", "start": "FCC lattice melted by 5000 mixed steps",
           "steps": args.drift_steps, "every": 1000,
           "definition": "least-squares slope of E = KE + PE, per 1e6 steps, relative to the mean |E|"}
    for prec, name in ((cavgpu.MIXED, "mixed"), (cavgpu.FP64, "fp64")):
        t0 = time.perf_counter()
        slope, dmax, e = nve_drift(cavgpu, p_eq, v_eq, typ, params, prec, args.drift_steps, every=1000, series=True)
        out[name] = {"drift_per_1e6_steps": slope, "max_rel_dE": dmax, "E_first": float(e[0]),
                     "E_last": float(e[-1]), "wall_s": time.perf_counter() - t0,
                     "E_every_10000": [float(x) for x in e[9::10]]}
    print(json.dumps(out), flush=True)


def time_e2e(cavgpu, torch, pos, vel, typ, params, precision, steps, **launch):
    """Through the C ABI with host buffers: pinned host arrays -> context + upload ->
    set-up -> K steps (thermo of every step read back) -> download of the final state,
    all timed.  Returns the rate, the bytes copied per step each way, and the wall
    time of each phase (the per-call fixed cost is everything but `steps_ms`)."""
    import numpy as np

    n = len(pos)
    hp = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    hv = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    ht = torch.empty(n, dtype=torch.int64, pin_memory=True).numpy()
    hp[:] = pos
    hv[:] = vel
    ht[:] = typ
    op = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    ov = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    oa = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    thermo = np.zeros((steps, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s = cavgpu.System(hp, hv, ht.view(np.uint64), params, precision=precision, **launch)
    t1 = time.perf_counter()
    s.setup()
    t2 = time.perf_counter()
    rc = cavgpu.lib().cavgpu_run(s._h, steps, 1, cavgpu._ptr(thermo))
    if rc:
        raise cavgpu.CavError(rc, "run")
    t3 = time.perf_counter()
    cavgpu.lib().cavgpu_download(s._h, cavgpu._ptr(op), cavgpu._ptr(ov), cavgpu._ptr(oa))
    t4 = time.perf_counter()
    s.close()
    h2d = n * (3 * 8 + 3 * 8 + 8)
    d2h = steps * 5 * 8 + n * 3 * 3 * 8
    phases = {"create_upload_ms": 1e3 * (t1 - t0), "setup_ms": 1e3 * (t2 - t1), "steps_ms": 1e3 * (t3 - t2),
              "download_ms": 1e3 * (t4 - t3)}
    return n * steps / (t4 - t0), h2d / steps, d2h / steps, phases


# ---------------------------------------------------------------------------
def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_under_torchrun(sys.argv[1:], args.gpus))
    ws, rank, local = dist_setup()
    if ws != args.gpus and rank == 0:
        print(f"bench.py: --gpus {args.gpus} but WORLD_SIZE {ws}; measuring {ws} ranks", file=sys.stderr)
    import numpy as np

    import workloads as W

    pos, vel, typ, params = W.lj_fluid((args.cells,) * 3, seed=1002)
    n = len(pos)
    workload = f"lj_fluid_{n}_atoms_nve"
    config = {"workload": workload, "atoms": n, "fcc_cells": [args.cells] * 3, "rho": 0.8442, "T": 1.44,
              "rc": 2.5, "skin": 0.3, "dt": 0.005, "integrator": "velocity_verlet_nve",
              "rebuild": "half-skin displacement", "replicas_per_gpu": 1,
              "l2": "inputs larger than L2 (the Verlet list alone is ~310 MB per step; L2 is 126 MB)"}

    if args.impl == "reference":
        if rank != 0:
            return
        # the K and W of this call, each step a full step of the 1,048,576-atom system
        # (~0.55 s on one core); beyond 200 timed steps the window is cut at 200
        steps = max(1, min(args.steps, 200))
        warm = min(args.warmup, 20)
        rate, secs = cpu_reference_rate(pos, vel, typ, params, steps, warm)
        sample = (f"{n} atoms, set-up + {warm} warm-up steps untimed, {steps} timed steps ({secs:.1f} s) of the "
                  "reference's serial cell-list path (oracle/cav_oracle.c); 1 core, 1 process, 1 MPI rank, "
                  f"{cpu_model()}")
        line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
                "steps": steps, "warmup": warm, "ms_per_step": 1e3 * secs / steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
                "cpu_baseline": {"value": rate, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample},
                "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch

    import cavgpu

    torch.cuda.set_device(local)
    sid = gpu_uuid()
    if args.drift_only:
        if rank == 0:
            drift_only(args, cavgpu, W, np)
        return

    # mixed precision (headline) and all-FP64, state resident in HBM
    tune = not args.no_tune
    sm, rm = time_device(cavgpu, torch, pos, vel, typ, params, cavgpu.MIXED, args.steps, args.warmup, ws, sid, tune)
    s64, r64 = time_device(cavgpu, torch, pos, vel, typ, params, cavgpu.FP64, max(args.steps // 4, 50),
                           min(args.warmup, 20), ws, sid, tune)
    ms_mixed = max_over_ranks(ws, rm["ms"])
    ms_fp64 = max_over_ranks(ws, r64["ms"])
    k64 = max(args.steps // 4, 50)
    value = ws * n * args.steps / (ms_mixed * 1e-3)
    value64 = ws * n * k64 / (ms_fp64 * 1e-3)

    # accuracy of the mixed form against FP64 at one thermalised state (the melted
    # fluid after the FP64 run; the initial lattice has zero net forces)
    p_eq, v_eq, _ = s64.state()
    sm.close()
    s64.close()
    f64 = cavgpu.System(p_eq, v_eq, typ, params, precision=cavgpu.FP64, **LAUNCH)
    f64.setup()
    fm = cavgpu.System(p_eq, v_eq, typ, params, precision=cavgpu.MIXED, **LAUNCH)
    fm.setup()
    a_ref, a_mix = f64.state()[2], fm.state()[2]
    t_ref, t_mix = f64.thermo(), fm.thermo()
    f64.close()
    fm.close()
    force_rms = float(np.sqrt(((a_mix - a_ref) ** 2).sum(1).mean() / (a_ref ** 2).sum(1).mean()))

    # NVE drift from an equilibrated fluid: the melted state relaxed 3000 more steps
    d64 = max(args.drift_steps // 4, 500) if args.drift_steps > 0 else 0
    if args.drift_steps > 0:
        eq = cavgpu.System(p_eq, v_eq, typ, params, precision=cavgpu.MIXED, **LAUNCH)
        eq.setup()
        eq.step(3000)
        p_eq, v_eq, _ = eq.state()
        eq.close()
    drift_m, dE_m = nve_drift(cavgpu, p_eq, v_eq, typ, params, cavgpu.MIXED, args.drift_steps)
    drift_64, dE_64 = nve_drift(cavgpu, p_eq, v_eq, typ, params, cavgpu.FP64, d64)

    tuned = rm["autotune"] or {}
    kern = {"segments": cavgpu.FORCE_SEGMENTS, "strided": cavgpu.FORCE_STRIDED}.get(tuned.get("force_kernel"),
                                                                                      cavgpu.FORCE_AUTO)
    spg = LAUNCH.get("steps_per_graph", tuned.get("steps_per_graph", 0))
    e2e_rate, h2d, d2h, phases = time_e2e(cavgpu, torch, pos, vel, typ, params, cavgpu.MIXED, args.steps,
                                          tpa=rm["tpa"], block=rm["block"], steps_per_graph=spg, force_kernel=kern)
    e2e_rate = ws * n * args.steps / max_over_ranks(ws, n * args.steps / e2e_rate)
    # the same call shape over a long window: the per-call fixed cost amortised
    long_steps = max(args.steps, 2000)
    e2e_long, _, _, phases_long = time_e2e(cavgpu, torch, pos, vel, typ, params, cavgpu.MIXED, long_steps,
                                           tpa=rm["tpa"], block=rm["block"], steps_per_graph=spg, force_kernel=kern)

    # roofline of the dominant kernel (mixed force kernel): algorithmic bytes per launch
    #   per atom: 4 * nbar list words + rel_i 16 + nnbr 4 + vel r/w 64 + acc r 32 (a_old) + acc w 32,
    #   and on the launches that also drift the next step: pos r/w 64 + pos_ref 32 + rel_ref 16
    #   + the next rel 16 = 128 more
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    peak_note = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    fused = fused_fraction(args.steps, rm["autotune"])
    bytes_per_atom = 4.0 * rm["nbar"] + 148.0 + 128.0 * fused
    launch_ms = rm["force_ms"] / max(rm["force_launches"], 1)
    achieved = bytes_per_atom * n / (launch_ms * 1e-3) / 1e9
    traffic = read_profile_traffic("lj_force_mixed_1M.md")
    # FP64 form: FP64-pipe roofline, FLOPs per atom = 8 n_list + 17 n_cut (n_cut = n_list (rc/ce)^3)
    fp64_peak, fp32_peak = cavgpu.measure_peaks()
    ncut = r64["nbar"] * (2.5 / 2.8) ** 3
    flops_atom = 8 * r64["nbar"] + 17 * ncut
    l64 = r64["force_ms"] / max(r64["force_launches"], 1)
    fp64_achieved = flops_atom * n / (l64 * 1e-3) / 1e12

    extra = None
    if not args.no_extra:
        extra = extra_workloads(cavgpu, torch, W, np, value / ws, ws, rank)

    cpu = None
    if rank == 0 and not args.no_cpu:
        rate, secs = cpu_reference_rate(pos, vel, typ, params, 20, 5)
        cpu = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{n} atoms, set-up + 5 warm-up steps untimed, 20 timed steps ({secs:.1f} s) of the "
                         "reference's serial cell-list path restated in oracle/cav_oracle.c; 1 core, 1 process, "
                         f"1 MPI rank, {cpu_model()}"}

    if rank != 0:
        return
    config.update({"fp64_value": value64, "mixed_over_fp64": value / value64, "fp64_steps": k64,
                   "rebuilds_in_timed_region": rm["rebuilds"], "mean_neighbours": rm["nbar"],
                   "threads_per_atom": rm["tpa"], "block": rm["block"], "capacity": rm["capacity"],
                   "autotune": rm["autotune"], "parallelism": f"replicas x{ws}"})
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_mixed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "mixed (f32 pair math, f64 state and reductions)",
        "data": "synthetic seeded FCC LJ fluid (no dataset exists for this path)", "config": config,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "kernel": "k_force<mixed>", "peak_source": peak_note,
                     "bytes_per_atom": bytes_per_atom, "launch_ms": launch_ms, "fused_launch_share": fused},
        "fp64": {"value": value64, "ms_per_step": ms_fp64 / k64, "kernel": "k_force<fp64>",
                 "roofline": {"bound": "fp64", "achieved": fp64_achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                              "frac": fp64_achieved / fp64_peak, "flops_per_atom": flops_atom, "launch_ms": l64,
                              "peak_source": "measured by cavgpu_measure_peaks (DFMA chains)"},
                 "clocks": r64["clocks"]},
        "accuracy": {"mixed_force_rms_rel": force_rms,
                     "mixed_pe_rel": abs(t_mix["pe"] - t_ref["pe"]) / abs(t_ref["pe"]),
                     "mixed_pressure_rel": abs(t_mix["pressure"] - t_ref["pressure"]) / abs(t_ref["pressure"]),
                     "nve_drift_per_1e6_steps": {"mixed": drift_m, "fp64": drift_64},
                     "nve_max_rel_dE": {"mixed": dE_m, "fp64": dE_64},
                     "drift_steps": {"mixed": args.drift_steps, "fp64": d64},
                     "drift_start": "melted fluid after the FP64 timed run, then 3000 mixed steps; signed "
                                    "least-squares slope of KE+PE sampled every 100 steps, per 1e6 steps, "
                                    "relative to the mean |E|"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_rate, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "phases_ms": phases,
                "fixed_ms": phases["create_upload_ms"] + phases["setup_ms"] + phases["download_ms"],
                "steady_value": n * args.steps / (phases["steps_ms"] * 1e-3),
                "long_window": {"steps": long_steps, "value": e2e_long, "phases_ms": phases_long}},
        "gpu_launches": rm["kernel_launches"],
        "clocks": rm["clocks"],
        "peaks": {"fp64_tflops": fp64_peak, "fp32_tflops": fp32_peak},
        "other_configs": extra,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
