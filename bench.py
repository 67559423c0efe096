#!/usr/bin/env python3
"""Benchmark of the GB300 nonbonded-force engine on the 98,304-site SPC water system.

Workload (one "step" = one complete force evaluation, frclong() + frcshort() of the
reference, src/frclong.c:20 and src/frcshort.c:20): 32,768 flexible SPC water molecules,
box 99.3 A, LJ + Ewald (alpha 0.3/A, real-space cutoff 10 A, kmax 24 per axis, spherical
ksqmax 576), harmonic bonds and angles; seeded synthetic coordinates (jittered lattice,
random orientations); mixed precision (FP32 pair arithmetic, FP64 accumulation).

metric  pair interactions per second: inter-molecular site pairs inside the cutoff
        (counted once) times steps, over the device time of the steps.
value   inputs resident in HBM (mg_compute_device); L2 (129 MB) flushed by a 256 MiB
        write before every step, each step timed alone with CUDA events on the stream the
        engine launches on.
e2e     the same through mg_compute with pinned host buffers: positions copied in and
        forces copied out inside the timed region.
Also reported: the plain-FP64 GPU path on the same workload; ns/day of the device-resident
Nose-Hoover RESPA integrator (mg_md_run; inner: bonded + pairs < 7 A, four 0.5 fs steps;
outer: 7-10 A shell + reciprocal, 2 fs) and the energy drift of an NVE run; batched HMC
of 512 Lennard-Jones replicas; the cost of the adjoint and Hessian-vector product; force
matching on 4096 waters (64 snapshots, loss + gradient, checked against the FP64 path and
central differences); 20,000 butane in a nanotube bundle with device-generated Tasos
tables (pair throughput, solid-fluid gather against HBM, ns/day, FP64 path); the roofline
of the dominant kernel and a CPU baseline of the reference algorithm: one full, unsampled
frclong()+frcshort() call of the oracle port on all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FP32_LANES_PER_SM = 128
# algorithmic work per unit: the fixed constants of the work model (perf/work_model.py)
from perf.work_model import (FLOP_K_F, FLOP_K_S, FLOP_KF_ROW, FLOP_KF_ROWKZ, FLOP_PAIR,  # noqa: E402
                             FLOP_SK_ROW, FLOP_SK_ROWKZ, SF_BYTES_PER_SITE, list_build_bytes,
                             neighbour_streaming_bytes)


def ewald_rows(kmax, ksqmax):
    """Rows (kx, ky) of the half-space k-vector set and the sum over rows of kzmax + 1
    (the |kz| values a row holds), as the engine enumerates them."""
    kx_max, ky_max, kz_max = kmax
    nrows = nkz = 0
    for kx in range(kx_max + 1):
        for ky in range(-ky_max, ky_max + 1):
            if kx == 0 and ky < 0:
                continue
            rem = ksqmax - kx * kx - ky * ky
            if rem < 0:
                continue
            m = 0
            while m + 1 <= kz_max and (m + 1) ** 2 <= rem:
                m += 1
            if kx == 0 and ky == 0 and m < 1:
                continue
            nrows += 1
            nkz += m + 1
    return nrows, nkz


def sk_tensor_flops(kmax, ksqmax, n, sites_per_block=1024, rows_per_tile=64, chunk=32):
    """FLOP the tensor-core S(k) pass (k_sk_mma) issues: rows sorted by kzmax (longest
    first) in tiles of 64, each tile an M = 128 x N = 2H GEMM (H = 16 if its longest row has
    kzmax < 16, else 32) over the sites of every block padded to whole 32-site chunks, three
    FP16 MMAs (hi*hi, hi*lo, lo*hi) per product."""
    kx_max, ky_max, kz_max = kmax
    kz = []
    for kx in range(kx_max + 1):
        for ky in range(-ky_max, ky_max + 1):
            if kx == 0 and ky < 0:
                continue
            rem = ksqmax - kx * kx - ky * ky
            if rem < 0:
                continue
            m = 0
            while m + 1 <= kz_max and (m + 1) ** 2 <= rem:
                m += 1
            if kx == 0 and ky == 0 and m < 1:
                continue
            kz.append(m)
    kz.sort(reverse=True)
    padded = sum(-(-min(sites_per_block, n - b) // chunk) * chunk for b in range(0, n, sites_per_block))
    flop = 0
    for t in range(0, len(kz), rows_per_tile):
        h = 16 if kz[t] + 1 <= 16 else 32
        flop += 3 * 2 * 128 * 2 * h * padded
    return flop


def kf_tensor_flops(kmax, ksqmax, n, sites_per_tile=128, rows_per_tile=64):
    """FLOP the tensor-core k-space force pass (k_kforce_mma) issues: rows sorted by kzmax
    (longest first) in tiles of 64, each tile an M = 128 (sites) x N = 256 (four sums per
    row) GEMM over K = 2 (kzmax + 1) rounded up to 16, for every 128-site tile, three FP16
    MMAs (hi*hi, hi*lo, lo*hi) per product."""
    kx_max, ky_max, kz_max = kmax
    kz = []
    for kx in range(kx_max + 1):
        for ky in range(-ky_max, ky_max + 1):
            if kx == 0 and ky < 0:
                continue
            rem = ksqmax - kx * kx - ky * ky
            if rem < 0:
                continue
            m = 0
            while m + 1 <= kz_max and (m + 1) ** 2 <= rem:
                m += 1
            if kx == 0 and ky == 0 and m < 1:
                continue
            kz.append(m)
    kz.sort(reverse=True)
    site_tiles = -(-n // sites_per_tile)
    flop = 0
    for t in range(0, len(kz), rows_per_tile):
        ksteps = -(-(2 * (kz[t] + 1)) // 16)
        flop += 3 * 2 * sites_per_tile * 4 * rows_per_tile * 16 * ksteps * site_tiles
    return flop


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="water_c2", choices=["water_c2", "water_c4", "water_c1"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-extras", action="store_true", help="skip FP64 path, RESPA and CPU baseline")
    ap.add_argument("--ref-slices", type=int, default=8,
                    help="reference arm: steps per full CPU call (each step one slice of it)")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the full-call CPU baseline")
    ap.add_argument("--md-dt-sweep", action="store_true",
                    help="print the NVE drift of the water system against the outer time step and exit")
    ap.add_argument("--nve-drift-scan", action="store_true",
                    help="only the NVE drift of the 216-water system at 0.5, 0.25 and 0.125 fs (20 ps each)")
    ap.add_argument("--nve-drift", action="store_true",
                    help="print a long small-step NVE drift run of the 216-water Wolf system on the mixed "
                         "path (with the power of its force error against the FP64 path) and exit")
    return ap.parse_args()


def max_over_ranks(dist, v, device):
    """The largest of the ranks' values, on every rank (a replica job takes as long as its
    slowest rank); v itself without a process group. device is where the collective's
    tensor lives: "cuda" under NCCL, "cpu" under gloo."""
    if dist is None:
        return float(v)
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, units_per_rank, ms):
    """Whole-job throughput: every rank processes units_per_rank per step (replicas, weak
    scaling) and a step takes ms milliseconds (the maximum over ranks)."""
    return world * units_per_rank / (ms * 1e-3)


def make_system(name):
    from mspms2_gb300 import configs
    return {"water_c2": configs.water_c2, "water_c4": configs.water_c4, "water_c1": configs.water_c1}[name]()


def pairs_in_cutoff(s):
    """Inter-molecular site pairs (neither GHOST_FULL) with r < cutoff, counted once."""
    from scipy.spatial import cKDTree
    q, g, mol = s.site_arrays()
    keep = g != 2
    pts = np.stack([s.x, s.y, s.z], 1)[keep]
    L = np.asarray(s.box, dtype=float)
    pts = pts - L * np.floor(pts / L)
    pts = np.minimum(pts, np.nextafter(L, 0))
    r = max(s.rcutoff, s.rcutoffelec)
    t = cKDTree(pts, boxsize=L)
    total = (int(t.count_neighbors(t, r)) - len(pts)) // 2
    intra = 0
    for sp in s.species:
        xyz = sp.template_xyz
        a = np.where(sp.ghost != 2)[0]
        d = np.linalg.norm(xyz[a][:, None] - xyz[a][None], axis=-1)
        intra += int(np.triu(d < r, 1).sum()) * sp.nmole
    return total - intra


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.file.read().splitlines():
            p = [v.strip() for v in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        self.file.close()
        os.unlink(self.file.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp32_peak_inputs(device, clk):
    """SM count read from the device and the SM clock ceiling sampled by nvidia-smi during
    the timed region (else MEASURED_PEAKS.json's sm_max_mhz) for the FP32 FMA-pipe peak:
    SMs x 128 lanes x 2 FLOP x clock. MEASURED_PEAKS.json holds no FP32 figure."""
    import torch
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    mhz, src = (clk or {}).get("sm_max_mhz"), "clocks.max.sm sampled during the timed region"
    if not mhz:
        mhz, src = measured_peaks().get("sm_max_mhz"), "MEASURED_PEAKS.json sm_max_mhz"
    if not mhz:
        mhz, src = 2070.0, "nominal 2070 MHz (no clock reading)"
    basis = (f"FP32 FMA pipe: {sms} SMs (read from the device) x 128 lanes x 2 FLOP x {mhz:.0f} MHz ({src}); "
             "MEASURED_PEAKS.json holds no FP32 figure")
    return sms, float(mhz), basis


def measured_peaks():
    try:
        with open(PEAKS_FILE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline(system, threads):
    """One full, unsampled evaluation of the reference algorithm on the host: the oracle
    port of src/frclong.c (orc_frclong_mt: the O(N^2) pair rows in ranges of equal pair count
    and the k-vectors dealt round robin over `threads` host threads, partial sums added in
    thread order) followed by src/frcshort.c (orc_frcshort, one thread); wall clock of each."""
    from oracle.pyoracle import Oracle
    o = Oracle(system)
    t0 = time.perf_counter()
    o.frclong_mt(threads)
    t1 = time.perf_counter()
    o.frcshort()
    t2 = time.perf_counter()
    return {"t_step_s": t2 - t0, "t_frclong_s": t1 - t0, "t_frcshort_s": t2 - t1, "threads": threads,
            "sample": f"one full unsampled frclong()+frcshort() call of the whole workload ({system.natom} sites, "
                      f"all pair rows and all k-vectors) on {threads} host thread(s); nothing extrapolated"}


def run_reference(args, rank):
    """The reference's CPU implementation of the path (the oracle port; the compiled
    reference does not exist on the GPU host) on all host threads. One step is slice k mod S
    of one full call (orc_frclong_mt slices: the k-th of S equal shares of the pair rows and
    the k-vectors numbered k mod S; slice 0 also runs the O(N) terms and frcshort), so S
    consecutive steps do one full call's work exactly once and every step is timed as run.
    S is picked so that a step takes a few seconds."""
    if rank != 0:
        return 0
    from oracle.pyoracle import Oracle
    system = make_system(args.workload)
    system.respa_split = 0.0
    npairs = pairs_in_cutoff(system)
    threads = host_threads()
    o = Oracle(system)
    S = max(1, args.ref_slices)

    def one(k):
        t0 = time.perf_counter()
        o.frclong_mt(threads, slice_=k % S, nslices=S)
        if k % S == 0:
            o.frcshort()
        return time.perf_counter() - t0

    for k in range(args.warmup):  # warm-up: slices of a finer partition (untimed)
        o.frclong_mt(threads, slice_=k % (4 * S), nslices=4 * S)
    t0 = time.perf_counter()
    ts = [one(k) for k in range(args.steps)]
    wall = time.perf_counter() - t0
    # pair interactions per second: each slice does 1/S of a full call's work
    value = npairs * len(ts) / S / sum(ts)
    full_calls = len(ts) // S
    full_s = [sum(ts[c * S:(c + 1) * S]) for c in range(full_calls)]
    sample = (f"each step is one of {S} slices of a full unsampled frclong()+frcshort() call ({system.natom} sites): "
              f"1/{S} of the pair rows (equal pair count) and every {S}th k-vector, on {threads} host threads; "
              f"{S} consecutive steps = one full call, timed in parts (nothing extrapolated)")
    line = {"impl": "reference", "metric": "pair_interactions_per_s", "value": value,
            "unit": "pair-interactions/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * statistics.mean(ts), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "sites": system.natom, "pairs_in_cutoff": npairs,
                       "slices_per_full_call": S},
            "full_call_s": full_s,
            "cpu_baseline": {"value": value, "unit": "pair-interactions/s", "cores": threads, "kind": "port",
                             "sample": sample, "host_cores": os.cpu_count()},
            "e2e": {"value": value, "unit": "pair-interactions/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line), flush=True)
    return 0


def md_extras(system, split_r, precision, device, steps=10, equil_steps=1000, nve_steps=500, fp64_steps=60):
    """ns/day of mg_md_run (NVT, vver_nh_3) and the energy drift of NVE runs (vver) on the
    workload, from seeded Maxwell-Boltzmann velocities at 298 K with zero momentum. The
    drift is taken after an NVT equilibration of equil_steps outer steps (the lattice start
    relaxes strongly): a linear fit of ukin + uinter + uintra over nve_steps outer steps on
    the mixed path, and over the first fp64_steps from the same state on both paths."""
    from mspms2_gb300.engine import Engine
    from mspms2_gb300.system import md_params, time_base
    s = system
    s.respa_split = split_r
    s.delt_fs, s.nstep_inner, s.treq_K = 2.0, 4, 298.0
    md = md_params(s)
    # Nose-Hoover masses for a 100 fs coupling time, Q = g T tau^2 (a fixed Q would couple
    # ever more stiffly as the system grows: Q = 1000 gives ~3 fs at 295k degrees of freedom)
    tau = 100.0 / time_base(s)
    md["qq"] = md["qqs"] = md["gg"] * md["treq"] * tau * tau
    m = np.concatenate([np.tile(sp.aw, sp.nmole) for sp in s.species])
    rng = np.random.default_rng(7)
    v = rng.normal(size=(3, s.natom)) * np.sqrt(md["treq"] / m)
    v -= (v * m).sum(1, keepdims=True) / m.sum()
    out = {"nh_tau_fs": 100.0}

    def keep(st):
        return {k: st[k] for k in ("ps", "ss", "pss", "sss")}

    with Engine(s, precision=precision, skin=1.0, device=device) as eng:
        md["scheme"] = 1
        pos, vel, st, _ = eng.md_run(2, md, v)  # warm-up: list, tables, solver
        t0 = time.perf_counter()
        pos, vel, st, log = eng.md_run(steps, md, vel, x=pos[0], y=pos[1], z=pos[2], state=keep(st))
        dt_wall = time.perf_counter() - t0
        out["scheme"] = "NVT Nose-Hoover RESPA (vver_nh_3), 4 x 0.5 fs inner + 2 fs outer"
        out["split_A"] = split_r
        out["steps"] = steps
        out["ms_per_outer_step"] = dt_wall / steps * 1e3
        out["ns_per_day"] = steps * 2.0e-6 / dt_wall * 86400.0
        out["tinst_K"] = [float(log[0, 8]), float(log[-1, 8])]
        pos, vel, st, log = eng.md_run(equil_steps, md, vel, x=pos[0], y=pos[1], z=pos[2], state=keep(st))
        out["equilibration"] = {"outer_steps": equil_steps, "tinst_K_end": float(log[-1, 8])}
        md["scheme"] = 0
        start = (pos.copy(), vel.copy())
        _, _, _, log = eng.md_run(nve_steps, md, vel, x=pos[0], y=pos[1], z=pos[2])
    with Engine(s, precision="fp64", skin=1.0, device=device) as e64:
        _, _, _, log64 = e64.md_run(fp64_steps, md, start[1], x=start[0][0], y=start[0][1], z=start[0][2])
    s.respa_split = 0.0

    def series(lg):
        return lg[:, 0] + lg[:, 1] + lg[:, 2]  # ukin + uinter + uintra (K)

    def drift(h):
        slope = float(np.polyfit(np.arange(len(h)) * 2.0, h, 1)[0])  # K per fs
        return slope * 1e6 / (md["treq"] * s.natom)
    h = series(log)
    out["nve"] = {"outer_steps": nve_steps, "ps": nve_steps * 2.0e-3,
                  "drift_kT_per_ns_per_atom": drift(h),
                  "rms_fluctuation_kT_per_atom": float(np.std(h)) / (md["treq"] * s.natom),
                  "window_steps": fp64_steps,
                  "window_drift_mixed": drift(h[:fp64_steps + 1]), "window_drift_fp64": drift(series(log64)),
                  "window_drift_of_mixed_minus_fp64": drift(h[:fp64_steps + 1] - series(log64))}
    out["note"] = ("device-resident: positions, velocities and thermostat scalars stay in HBM; timed with the "
                   "wall clock around mg_md_run (host copies of the start and end included); drift from a "
                   "linear fit of ukin + uinter + uintra over the NVE run after the NVT equilibration")
    return out


def c1_extras(device, steps=1000):
    """The small CPU-runnable configuration: 216 SPC/Fw waters (648 sites), Wolf alpha 0.2/A,
    Rc 9 A, Nose-Hoover NVT (vver_nh_3) at 298 K, 0.5 fs, 1000 steps, from one set of
    seeded velocities: on the device through mg_md_run (both precisions), and on one host
    core through the oracle port of the same integrator (orc_md_run; the reference is
    single-threaded). Wall clock around each whole run; the FP64 device run and the CPU
    run are compared at the end of the trajectory."""
    from mspms2_gb300 import configs
    from mspms2_gb300.engine import Engine
    from mspms2_gb300.system import md_params, time_base
    from oracle.pyoracle import Oracle
    s = configs.water_c1()
    s.delt_fs, s.nstep_inner, s.treq_K = 0.5, 1, 298.0
    md = md_params(s)
    md["scheme"] = 1
    tau = 100.0 / time_base(s)
    md["qq"] = md["qqs"] = md["gg"] * md["treq"] * tau * tau
    m = np.concatenate([np.tile(sp.aw, sp.nmole) for sp in s.species])
    v = np.random.default_rng(11).normal(size=(3, s.natom)) * np.sqrt(md["treq"] / m)
    v -= (v * m).sum(1, keepdims=True) / m.sum()
    out = {"workload": "water_c1 (216 SPC/Fw, Wolf, NVT 298 K, 0.5 fs)", "steps": steps}
    ends = {}
    for prec in ("mixed", "fp64"):
        with Engine(s, precision=prec, device=device) as eng:
            eng.md_run(5, md, v)  # warm-up: list, solver, graph capture
            t0 = time.perf_counter()
            pos, _, _, lg = eng.md_run(steps, md, v)
            dt = time.perf_counter() - t0
        ends[prec] = (pos, lg)
        out[f"gpu_{prec}"] = {"wall_s": dt, "ms_per_step": dt / steps * 1e3,
                              "ns_per_day": steps * 0.5e-6 / dt * 86400.0}
    t0 = time.perf_counter()
    pos_c, _, _, lg_c = Oracle(s).md_run(steps, md, v)
    dt = time.perf_counter() - t0
    out["cpu_port_1_thread"] = {"wall_s": dt, "ms_per_step": dt / steps * 1e3, "ns_per_day": steps * 0.5e-6 / dt * 86400.0}
    pos64, lg64 = ends["fp64"]
    out["fp64_gpu_vs_cpu_end"] = {"max_abs_position_diff_A": float(np.abs(pos64 - pos_c).max()),
                                  "total_energy_rel_diff": float(abs((lg64[-1, :3].sum() - lg_c[-1, :3].sum()) /
                                                                      lg_c[-1, :3].sum()))}
    out["gpu_mixed_over_cpu"] = out["cpu_port_1_thread"]["wall_s"] / out["gpu_mixed"]["wall_s"]
    out["note"] = ("wall clock of the whole run, host copies of the start and end state included; the CPU run is "
                   "the restated vver_nh_3 with frclong/frcshort of the oracle on one host core")
    return out


def nve_drift_scan(device=0, ps=20.0, cases=((0.5, "mixed"), (0.25, "mixed"), (0.125, "mixed"), (0.125, "fp64"))):
    """NVE drift against the time step on the 216-water Wolf system: for each (step, path),
    1 ps of Nose-Hoover NVT at 298 K from seeded velocities, then `ps` of velocity-Verlet NVE;
    drift = slope of ukin + uinter + uintra. Integration error shows as drift ~ dt^2."""
    from mspms2_gb300 import configs
    from mspms2_gb300.engine import Engine
    from mspms2_gb300.system import md_params, time_base
    out = []
    for dt_fs, prec in cases:
        steps = int(ps * 1e3 / dt_fs)
        s = configs.water_c1()
        s.delt_fs, s.nstep_inner, s.treq_K = dt_fs, 1, 298.0
        md = md_params(s)
        tau = 100.0 / time_base(s)
        md["qq"] = md["qqs"] = md["gg"] * md["treq"] * tau * tau
        m = np.concatenate([np.tile(sp.aw, sp.nmole) for sp in s.species])
        rng = np.random.default_rng(11)
        v = rng.normal(size=(3, s.natom)) * np.sqrt(md["treq"] / m)
        v -= (v * m).sum(1, keepdims=True) / m.sum()
        with Engine(s, precision=prec, device=device) as eng:
            md["scheme"] = 1
            pos, vel, _, _ = eng.md_run(int(1000 / dt_fs), md, v)
            md["scheme"] = 0
            _, _, _, lg = eng.md_run(steps, md, vel, x=pos[0], y=pos[1], z=pos[2])
        h = lg[:, 0] + lg[:, 1] + lg[:, 2]
        slope = float(np.polyfit(np.arange(len(h)) * dt_fs, h, 1)[0])
        fl = float(np.std(h)) / (md["treq"] * s.natom)
        out.append({"dt_fs": dt_fs, "precision": prec, "ps": ps, "drift_kT_per_ns_per_atom":
                    slope * 1e6 / (md["treq"] * s.natom), "rms_fluctuation_kT_per_atom": fl,
                    "resolution_kT_per_ns_per_atom": fl / (ps * 1e-3)})
    return {"workload": "water_c1 (216 SPC/Fw, Wolf)", "integrator": "velocity Verlet (vver), NVE", "runs": out}


def drift_fit(t_ns, h, natom_kT):
    """Linear drift of an energy series h(t) in kT/ns/atom with its standard error, the
    residuals' autocorrelation taken into account (integrated autocorrelation time up to
    the first zero of the autocorrelation; effective samples N dt / 2 tau), and the
    conservative resolution (RMS fluctuation / duration)."""
    t = np.asarray(t_ns, dtype=float)
    y = np.asarray(h, dtype=float) / natom_kT
    A = np.stack([t, np.ones_like(t)], 1)
    coef, *_ = np.linalg.lstsq(A, y, rcond=None)
    res = y - A @ coef
    r = res - res.mean()
    n = len(r)
    f = np.fft.rfft(r, 2 * n)
    ac = np.fft.irfft(f * np.conj(f))[:n]
    ac = ac / ac[0]
    cut = int(np.argmax(ac <= 0.0)) if np.any(ac <= 0.0) else n
    tau = 0.5 + float(ac[1:max(cut, 1)].sum())  # in samples
    neff = max(n / (2.0 * tau), 2.0)
    span = t[-1] - t[0]
    se = float(np.std(res)) * np.sqrt(12.0 / neff) / span
    return {"drift_kT_per_ns_per_atom": float(coef[0]), "stderr_kT_per_ns_per_atom": se,
            "rms_fluctuation_kT_per_atom": float(np.std(y)), "resolution_rms_over_span": float(np.std(y)) / span,
            "autocorrelation_samples": tau, "ns": float(span)}


def nve_drift(device=0, dt_fs=0.25, equil_steps=4000, steps=7_000_000, chunk=4000, every=40):
    """Energy drift of plain velocity-Verlet NVE on the 216-water Wolf system (648 sites,
    rc 9 A, alpha 0.2/A) at a small step, long enough to resolve 1e-4 kT/ns/atom, and the
    mixed path's own share of it. One state is equilibrated by Nose-Hoover NVT at 298 K (tau
    100 fs); then `steps` NVE steps on the mixed path run in chunks of the graph-replayed
    integrator (mg_md_run), the total energy sampled every `every` steps and fitted with an
    autocorrelation-aware standard error. At the end of every chunk the power of the mixed
    forces' error at that state, P = sum_i v_i . (F_mixed(x) - F_FP64(x)), is taken from a
    mixed and an FP64 context: its mean is the rate at which the mixed path's force error
    changes the total energy (the rest of the drift is the integrator's and the model's,
    the same on both paths), with a standard error from the spread of P over the chunks."""
    from mspms2_gb300 import configs
    from mspms2_gb300.engine import Engine
    from mspms2_gb300.system import md_params, time_base
    s = configs.water_c1()
    s.delt_fs, s.nstep_inner, s.treq_K = dt_fs, 1, 298.0
    md = md_params(s)
    tau = 100.0 / time_base(s)
    md["qq"] = md["qqs"] = md["gg"] * md["treq"] * tau * tau
    m = np.concatenate([np.tile(sp.aw, sp.nmole) for sp in s.species])
    rng = np.random.default_rng(11)
    v = rng.normal(size=(3, s.natom)) * np.sqrt(md["treq"] / m)
    v -= (v * m).sum(1, keepdims=True) / m.sum()
    natom_kT = md["treq"] * s.natom
    per_ns = 1.0e6 / time_base(s)  # reduced time units in one ns
    out = {"workload": "water_c1 (216 SPC/Fw, Wolf)", "dt_fs": dt_fs, "integrator": "velocity Verlet (vver), NVE",
           "sampled_every_steps": every, "power_samples_every_steps": chunk}
    t, h, power, fnorm = [], [], [], []
    with Engine(s, precision="mixed", device=device) as eng, Engine(s, precision="fp64", device=device) as e64:
        md["scheme"] = 1
        pos, vel, _, _ = eng.md_run(equil_steps, md, v)
        t0 = time.perf_counter()
        done = 0
        while done < steps:
            k = min(chunk, steps - done)
            pos, vel, _, lg = eng.md_run(k, dict(md, scheme=0), vel, x=pos[0], y=pos[1], z=pos[2])
            e = lg[:, 0] + lg[:, 1] + lg[:, 2]
            idx = np.arange(0 if done == 0 else every, k + 1, every)
            t.append((done + idx) * dt_fs * 1e-6)
            h.append(e[idx])
            done += k
            fl, fs, _ = eng.compute(pos[0], pos[1], pos[2])
            gl, gs, _ = e64.compute(pos[0], pos[1], pos[2])
            df = (fl + fs) - (gl + gs)
            power.append(float((vel * df).sum()))
            fnorm.append(float(np.linalg.norm(df) / np.linalg.norm(gl + gs)))
        wall = time.perf_counter() - t0
    fit = drift_fit(np.concatenate(t), np.concatenate(h), natom_kT)
    p = np.asarray(power) * per_ns / natom_kT
    out.update({"mixed": dict(fit, steps=steps, wall_s=wall),
                "mixed_force_error_power": {
                    "drift_kT_per_ns_per_atom": float(p.mean()),
                    "stderr_kT_per_ns_per_atom": float(p.std(ddof=1) / np.sqrt(len(p))),
                    "samples": len(p), "rms_rel_force_err": float(np.sqrt(np.mean(np.square(fnorm))))}})
    return out


def md_dt_sweep(precision="mixed", device=0, equil_steps=1000, ps=1.0):
    """NVE energy drift of the water system against the outer time step, from one state
    equilibrated by Nose-Hoover NVT (2 fs outer step, tau 100 fs): RESPA 2 fs / 4 x 0.5 fs,
    1 fs / 2 x 0.5 fs and plain velocity Verlet at 0.5 fs, each over `ps` picoseconds."""
    from mspms2_gb300 import configs
    from mspms2_gb300.engine import Engine
    from mspms2_gb300.system import md_params, time_base
    s = configs.water_c2()
    s.delt_fs, s.nstep_inner, s.treq_K = 2.0, 4, 298.0
    md = md_params(s)
    tau = 100.0 / time_base(s)
    md["qq"] = md["qqs"] = md["gg"] * md["treq"] * tau * tau
    m = np.concatenate([np.tile(sp.aw, sp.nmole) for sp in s.species])
    rng = np.random.default_rng(7)
    v = rng.normal(size=(3, s.natom)) * np.sqrt(md["treq"] / m)
    v -= (v * m).sum(1, keepdims=True) / m.sum()
    out = {"workload": "water_c2", "precision": precision, "equilibration_outer_steps": equil_steps}
    with Engine(s, precision=precision, skin=1.0, device=device) as eng:
        md["scheme"] = 1
        pos, vel, st, log = eng.md_run(equil_steps, md, v)
        out["T_after_equilibration_K"] = float(log[-1, 8])
        runs = []
        for outer_fs, inner in [(2.0, 4), (1.0, 2), (0.5, 1)]:
            mm = dict(md, scheme=0, delt=outer_fs / time_base(s), nstep_inner=inner)
            n = int(round(ps * 1000.0 / outer_fs))
            _, _, _, lg = eng.md_run(n, mm, vel, x=pos[0], y=pos[1], z=pos[2])
            h = lg[:, 0] + lg[:, 1] + lg[:, 2]
            slope = float(np.polyfit(np.arange(len(h)) * outer_fs, h, 1)[0])
            runs.append({"outer_fs": outer_fs, "inner_steps": inner, "steps": n,
                         "drift_kT_per_ns_per_atom": slope * 1e6 / (md["treq"] * s.natom),
                         "rms_fluctuation_kT_per_atom": float(np.std(h)) / (md["treq"] * s.natom)})
        out["nve"] = runs
    return out


def hmc_extras(device, nrep=512, nmoves=2, seed=2024):
    """Batched HMC (mg_hmc_batch) on nrep Lennard-Jones replicas with seeded sizes drawn
    uniformly from 200..5000 atoms (rho* 0.8, T* 1, rc 2.5 sigma, jittered FCC, 10-step
    trajectories at dt* 0.005): HMC trajectories per second of the whole batch."""
    from mspms2_gb300 import configs
    from mspms2_gb300.engine import hmc_batch
    rng = np.random.default_rng(seed)
    sizes = rng.integers(200, 5001, size=nrep)
    reps = [configs.lj_replica(int(n), seed=seed + i) for i, n in enumerate(sizes)]
    natom = [r.natom for r in reps]
    box = [float(r.box[0]) for r in reps]
    x, y, z = (np.concatenate([getattr(r, k) for r in reps]) for k in "xyz")
    hp = dict(eps=1.0, sigma=1.0, rcutoff=2.5, mass=1.0, treq=1.0, delt=0.005, nstep_md=10, seed=seed, rescale=0,
              nconstraint=0)
    hmc_batch(hp, natom, box, x, y, z, 1, device=device)  # warm-up
    t0 = time.perf_counter()
    _, _, _, acc, _, _ = hmc_batch(hp, natom, box, x, y, z, nmoves, move0=1, device=device)
    dt_wall = time.perf_counter() - t0
    steps = nrep * nmoves * 10
    return {"replicas": nrep, "atoms": int(sum(natom)), "moves_per_replica": nmoves,
            "trajectories_per_s": nrep * nmoves / dt_wall, "atom_steps_per_s": float(sum(natom)) * nmoves * 10 / dt_wall,
            "acceptance": float(acc.sum()) / (nrep * nmoves), "wall_s": dt_wall, "md_steps": steps,
            "note": "one persistent launch per call (host copies of all replicas included); Maxwell-Boltzmann "
                    "momenta without rescaling; FP32 pair forces, FP64 energies and Metropolis test"}


def siman_batch_extras(device, nrep=512, n_tries=25, seed=2024):
    """Batched simulated annealing (mg_siman_batch) of the same nrep Lennard-Jones replicas
    as hmc_extras (200..5000 atoms, rho* 0.8, rc 2.5 sigma), annealed from T* = 2 to below
    T* = 1 by T /= 1.3 (4 stages, as 600 K -> 300 K in the reference's siman), n_tries
    Nose-Hoover steps at dt* 0.005 per stage: replica-stages and atom-steps per second of
    the whole batch."""
    from mspms2_gb300 import configs
    from mspms2_gb300.engine import siman_batch
    rng = np.random.default_rng(seed)
    sizes = rng.integers(200, 5001, size=nrep)
    reps = [configs.lj_replica(int(n), seed=seed + i) for i, n in enumerate(sizes)]
    natom = [r.natom for r in reps]
    box = [float(r.box[0]) for r in reps]
    x, y, z = (np.concatenate([getattr(r, k) for r in reps]) for k in "xyz")
    sp = dict(eps=1.0, sigma=1.0, rcutoff=2.5, mass=1.0, delt=0.005, qq=50.0, qqs=50.0, t_initial=2.0, t_min=1.0,
              mu_t=1.3, n_tries=n_tries, max_stages=8, seed=seed, nconstraint=0)
    siman_batch(dict(sp, n_tries=1), natom, box, x, y, z, device=device)  # warm-up
    t0 = time.perf_counter()
    _, _, _, log = siman_batch(sp, natom, box, x, y, z, device=device)
    dt_wall = time.perf_counter() - t0
    nst = log.shape[1]
    return {"replicas": nrep, "atoms": int(sum(natom)), "stages": nst, "steps_per_stage": n_tries,
            "replica_stages_per_s": nrep * nst / dt_wall,
            "atom_steps_per_s": float(sum(natom)) * nst * n_tries / dt_wall, "wall_s": dt_wall,
            "final_tinst_mean": float(log[:, -1, 4].mean()), "final_T": float(log[0, -1, 0]),
            "note": "one persistent launch per call (host copies of all replicas included); per stage velinit "
                    "at T and n_tries vver_nh_3 steps; FP32 pair forces, FP64 thermostat and energies"}


def adjoint_extras(system, precision, device, reps=3):
    """Derivatives on the bench workload through the host API (positions and vectors in
    host memory, copies included): one long-force evaluation (mg_compute, MG_TERMS_LONG),
    the parameter adjoint (mg_adjoint_params, which runs that evaluation first) and the
    Hessian-vector product (mg_adjoint_hvp, likewise). Wall-clock milliseconds per call."""
    from mspms2_gb300.engine import TERMS_LONG, Engine
    n = system.natom
    rng = np.random.default_rng(17)
    g = rng.standard_normal((3, n))
    eng = Engine(system, precision=precision, device=device)
    try:
        eng.compute(terms=TERMS_LONG)
        eng.adjoint_params(g)
        eng.hessian_vector(g)

        def wall(fn):
            ts = []
            for _ in range(reps):
                t0 = time.perf_counter()
                fn()
                ts.append((time.perf_counter() - t0) * 1e3)
            return statistics.median(ts)

        t_f = wall(lambda: eng.compute(terms=TERMS_LONG))
        t_a = wall(lambda: eng.adjoint_params(g))
        t_h = wall(lambda: eng.hessian_vector(g))
        nclass = sum(t.natom for t in system.species)
    finally:
        eng.close()
    return {"long_forces_ms": t_f, "adjoint_params_ms": t_a, "hvp_ms": t_h,
            "adjoint_over_forces": t_a / t_f, "hvp_over_forces": t_h / t_f, "site_classes": nclass,
            "note": "host API wall time, median of 3; each derivative call includes its forward evaluation"}


def force_matching_extras(device, nsnap=64, stride=4, seed=2024):
    """Force matching on 4096 SPC/Fw waters (12,288 sites, Ewald alpha 0.3, rc 10 A, kmax 12):
    64 snapshots of an FP64 Nose-Hoover trajectory at 298 K (one every 4 steps of 0.5 fs from
    the seeded lattice); targets = FP64 long forces at eps_OO, sigma_OO, q_O perturbed by 2%
    Gaussian noise with q_H = -q_O/2; loss = mean squared force error over all snapshots.
    Times one loss + gradient evaluation over the 64 snapshots (mg_force_match per snapshot,
    host arrays) on the mixed and the FP64 path, and checks the gradient in (eps_O, sigma_O,
    q_O) against the FP64 path and against central differences of the FP64 loss
    (h = 1e-4 relative)."""
    from mspms2_gb300 import configs
    from mspms2_gb300.engine import TERMS_LONG, Engine
    from mspms2_gb300.system import md_params
    s = configs.water_c4(seed)
    s.delt_fs, s.nstep_inner, s.treq_K = 0.5, 1, 298.0
    md = md_params(s)
    md["scheme"] = 1
    m = np.concatenate([np.tile(sp.aw, sp.nmole) for sp in s.species])
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(3, s.natom)) * np.sqrt(md["treq"] / m)
    v -= (v * m).sum(1, keepdims=True) / m.sum()
    scale = 1.0 / (3 * s.natom * nsnap)

    def tied(base, p):
        e, sg, q = (a.copy() for a in base)
        e[0], sg[0] = p[0], p[1]
        q[:] = [p[2], -p[2] / 2, -p[2] / 2]
        return e, sg, q

    def fm_total(eng, snaps, targets):
        loss, g = 0.0, np.zeros(3)
        for x, t in zip(snaps, targets):
            li, (ge, gs, gq) = eng.force_match(t, scale=scale, x=x[0], y=x[1], z=x[2])
            loss += li
            g += [ge[0], gs[0], gq[0] - 0.5 * (gq[1] + gq[2])]
        return loss, g

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    snaps, targets = [], []
    with Engine(s, precision="fp64", skin=1.0, device=device) as e64:
        pos, vel, st = np.stack([s.x, s.y, s.z]), v, None
        for _ in range(nsnap):
            state = None if st is None else {k: st[k] for k in ("ps", "ss", "pss", "sss")}
            pos, vel, st, _ = e64.md_run(stride, md, vel, x=pos[0], y=pos[1], z=pos[2], state=state)
            snaps.append(pos.copy())
        base = list(e64.class_params())
        p0 = np.array([base[0][0], base[1][0], base[2][0]])
        p_tgt = p0 * (1 + 0.02 * np.random.default_rng(seed + 1).standard_normal(3))
        e64.set_class_params(*tied(base, p_tgt))
        targets = [e64.compute(*x, terms=TERMS_LONG)[0] for x in snaps]
        e64.set_class_params(*base)
        fm_total(e64, snaps[:1], targets[:1])
        t0 = time.perf_counter()
        l64, g64 = fm_total(e64, snaps, targets)
        t64 = time.perf_counter() - t0

        def loss64(p):
            e64.set_class_params(*tied(base, p))
            return scale * sum(float(np.sum((e64.compute(*x, terms=TERMS_LONG)[0] - t) ** 2))
                               for x, t in zip(snaps, targets))
        fd = np.zeros(3)
        for k in range(3):
            h = 1e-4 * abs(p0[k])
            pp, pm = p0.copy(), p0.copy()
            pp[k] += h
            pm[k] -= h
            fd[k] = (loss64(pp) - loss64(pm)) / (2 * h)
        e64.set_class_params(*base)
    with Engine(s, precision="mixed", skin=1.0, device=device) as emx:
        fm_total(emx, snaps[:2], targets[:2])
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            lmx, gmx = fm_total(emx, snaps, targets)
            ts.append(time.perf_counter() - t0)
        tmx = statistics.median(ts)
    return {"workload": "water_c4 force matching", "sites": s.natom, "snapshots": nsnap,
            "ms_per_gradient": tmx * 1e3, "snapshots_per_s": nsnap / tmx, "fp64_ms_per_gradient": t64 * 1e3,
            "mixed_over_fp64": t64 / tmx, "loss": lmx, "loss_fp64": l64,
            "grad_eps_sigma_qO": gmx.tolist(), "grad_rel_err_vs_fp64": rel(gmx, g64),
            "grad_fp64_rel_err_vs_central_diff": rel(g64, fd), "grad_mixed_rel_err_vs_central_diff": rel(gmx, fd),
            "note": "one mg_force_match per snapshot (forward + adjoint, host arrays, copies included); "
                    "gradient in (eps_OO, sigma_OO, q_O) with q_H = -q_O/2; central differences h = 1e-4 relative"}


def siman_batch_contexts(eng, s, md, sc, pos, nrep, device):
    """nrep annealing runs of the C5 system side by side on one GPU: the context eng and
    nrep - 1 more that use its Tasos tables (mg_sf_tasos_share), each on its own stream and
    driven by its own host thread, replica r with seed sc.seed + r. Reports the wall time of
    the batch against nrep runs one after another (the single run timed just before)."""
    import threading
    from mspms2_gb300.engine import Engine
    engs = [eng]
    for _ in range(nrep - 1):
        e = Engine(s, precision="mixed", device=device)
        e.sf_tasos_share(eng)
        engs.append(e)
    warm = dict(sc, n_tries=1, t_min=sc["t_initial"] * 0.999, max_stages=2)
    logs = [None] * nrep

    def work(r, schedule):
        logs[r] = engs[r].siman_run(md, dict(schedule, seed=sc["seed"] + r), x=pos[0], y=pos[1], z=pos[2])[3]

    def batch(schedule):
        th = [threading.Thread(target=work, args=(r, schedule)) for r in range(nrep)]
        t0 = time.perf_counter()
        for t in th:
            t.start()
        for t in th:
            t.join()
        return time.perf_counter() - t0

    batch(warm)
    wall = batch(sc)
    t0 = time.perf_counter()
    work(1, sc)
    solo = time.perf_counter() - t0
    for e in engs[1:]:
        e.close()
    steps = sum(len(lg) for lg in logs) * sc["n_tries"]
    return {"replicas": nrep, "form": "one context per replica, each on its own stream and host thread (not one launch)",
            "tables": "one copy shared by all contexts (mg_sf_tasos_share)",
            "wall_s": wall, "solo_wall_s": solo, "outer_steps": steps,
            "ms_per_outer_step": wall / steps * 1e3, "speedup_over_sequential": nrep * solo / wall,
            "stages": [int(len(lg)) for lg in logs]}


def c5_extras(device, steps=10, warmup=3, md_steps=5, fp64=True, siman_tries=10, replicas=8):
    """United-atom n-butane in a bundle of 7 (11,11) nanotubes (80,000 sites, LJ rc 14 A,
    Tasos solid-fluid tables at 0.1 A over the 127 x 127 A bundle cell, generated on the
    device): force steps timed like the headline (device-resident positions, L2 flushed,
    CUDA events), the solid-fluid gather against the HBM roofline (64 FP32 table values,
    256 B, per site), ns/day of Nose-Hoover RESPA (2 fs outer, 4 x 0.5 fs inner with the
    bonded terms), the reference's simulated annealing 600 K -> 300 K on the system, and the
    plain-FP64 path on the same system."""
    import torch
    from mspms2_gb300 import configs
    from mspms2_gb300.engine import TERMS_ALL, Engine
    from mspms2_gb300.system import md_params, time_base
    s, tubes = configs.butane_in_tube_bundle()
    per = tubes["period"]
    nx, ny, nz = configs.C5_TASOS_NODES
    h = configs.c5_tasos_spacing(tubes)

    def spec(sig, eps):
        return configs.c5_tasos_spec(tubes, sig, eps)

    n = s.natom
    stream = torch.cuda.current_stream()
    pos = torch.tensor(np.stack([s.x, s.y, s.z]), dtype=torch.float64, device="cuda")
    fl = torch.empty((3, n), dtype=torch.float64, device="cuda")
    fs = torch.empty((3, n), dtype=torch.float64, device="cuda")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    ptrs = (pos[0].data_ptr(), pos[1].data_ptr(), pos[2].data_ptr())
    out = {"workload": "butane_tube_bundle", "sites": n, "molecules": s.nmole, "rc_A": s.rcutoff,
           "tasos_nodes_per_table": nx * ny * nz, "tasos_spacing_A": [h[0], h[1], h[2]]}

    def timed(eng, k):
        eng.set_stream(stream.cuda_stream)
        for _ in range(warmup):
            eng.compute_device(*ptrs, fl.data_ptr(), fs.data_ptr(), TERMS_ALL)
        ts = []
        for i in range(k):
            flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            eng.compute_device(*ptrs, fl.data_ptr(), fs.data_ptr(), TERMS_ALL)
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.mean(ts)

    with Engine(s, precision="mixed", device=device) as eng:
        t0 = time.perf_counter()
        eng.sf_tasos_generate(1, spec(3.75, 98.0), nx, ny, nz, h, per)
        eng.sf_tasos_generate(2, spec(3.95, 46.0), nx, ny, nz, h, per)
        out["table_generation_s"] = time.perf_counter() - t0
        ms = timed(eng, steps)
        st = eng.stats()
        npairs = st["pairs_within_cutoff"]
        eng.set_timing(True)
        flush.fill_(1.0)
        eng.compute_device(*ptrs, fl.data_ptr(), fs.data_ptr(), TERMS_ALL)
        torch.cuda.synchronize()
        kms = eng.stats()["kernel_ms"]
        eng.set_timing(False)
        f32 = torch.cat([fl, fs]).clone()
        # ns/day of the RESPA integrator from seeded Maxwell-Boltzmann velocities at 300 K
        s.delt_fs, s.nstep_inner = 2.0, 4
        md = md_params(s)
        md["scheme"] = 1
        tau = 100.0 / time_base(s)
        md["qq"] = md["qqs"] = md["gg"] * md["treq"] * tau * tau
        m = np.concatenate([np.tile(sp.aw, sp.nmole) for sp in s.species])
        v = np.random.default_rng(5).normal(size=(3, n)) * np.sqrt(md["treq"] / m)
        v -= (v * m).sum(1, keepdims=True) / m.sum()
        p1, v1, st1, _ = eng.md_run(1, md, v)
        t0 = time.perf_counter()
        eng.md_run(md_steps, md, v1, x=p1[0], y=p1[1], z=p1[2], state={k: st1[k] for k in ("ps", "ss", "pss", "sss")})
        dt_md = time.perf_counter() - t0
        # the reference's simulated annealing on this system (mg_siman_run): T = 600 K / 1.3^k
        # until the first stage below 300 K, siman_tries RESPA outer steps per stage
        sc = dict(t_initial=600.0 / s.epsilon_base, t_min=300.0 / s.epsilon_base, mu_t=1.3, n_tries=siman_tries,
                  max_stages=8, seed=2024)
        eng.siman_run(md, dict(sc, n_tries=1, t_min=599.0 / s.epsilon_base, max_stages=2), x=p1[0], y=p1[1],
                      z=p1[2])  # warm-up: two stages of one step
        t0 = time.perf_counter()
        _, _, _, slog = eng.siman_run(md, sc, x=p1[0], y=p1[1], z=p1[2])
        dt_si = time.perf_counter() - t0
        batch = siman_batch_contexts(eng, s, md, sc, p1, replicas, device) if replicas > 1 else None
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    nsf = n  # every butane site is of ghost type NONE
    sf_gbs = nsf * SF_BYTES_PER_SITE / (kms[5] * 1e-3) / 1e9 if kms[5] > 0 else None
    out.update({"ms_per_step": ms, "pairs_in_cutoff": npairs, "value": npairs / (ms * 1e-3),
                "unit": "pair-interactions/s",
                "stage_ms": {"list": kms[0], "pair": kms[1], "intra_bonded": kms[2], "solid_fluid": kms[5],
                             "total": kms[7]},
                "sf_gather": {"bound": "hbm", "bytes_per_site": int(SF_BYTES_PER_SITE), "achieved_gbs": sf_gbs, "peak_gbs": hbm,
                              "frac": (sf_gbs / hbm) if (sf_gbs and hbm) else None,
                              "peak_basis": "of measured (MEASURED_PEAKS.json hbm_gbs)"},
                "md": {"scheme": "NVT Nose-Hoover RESPA, 4 x 0.5 fs inner (bonded) + 2 fs outer", "steps": md_steps,
                       "ms_per_outer_step": dt_md / md_steps * 1e3,
                       "ns_per_day": md_steps * 2.0e-6 / dt_md * 86400.0},
                "siman": {"schedule": "600 K / 1.3^k to the first stage below 300 K (the reference's siman)",
                          "stages": int(len(slog)), "steps_per_stage": siman_tries,
                          "T_K": [float(t) * s.epsilon_base for t in slog[:, 0]],
                          "tinst_K_end_of_stage": [float(t) * s.epsilon_base for t in slog[:, 5]],
                          "wall_s": dt_si, "ms_per_outer_step": dt_si / (len(slog) * siman_tries) * 1e3,
                          "note": "one system through the engine; replicas of this size run as separate "
                                  "contexts sharing one copy of the tables (siman_batch), not one launch"},
                "siman_batch": batch})
    if fp64:
        with Engine(s, precision="fp64", device=device) as e64:
            t0 = time.perf_counter()
            e64.sf_tasos_generate(1, spec(3.75, 98.0), nx, ny, nz, h, per)
            e64.sf_tasos_generate(2, spec(3.95, 46.0), nx, ny, nz, h, per)
            t_gen64 = time.perf_counter() - t0
            ms64 = timed(e64, 3)
            f64 = torch.cat([fl, fs]).clone()
        err = float(torch.linalg.vector_norm(f32 - f64) / torch.linalg.vector_norm(f64))
        out["fp64_path"] = {"ms_per_step": ms64, "mixed_over_fp64": ms64 / ms, "rms_rel_force_err_mixed_vs_fp64": err,
                            "table_generation_s": t_gen64}
    return out


def run_ours(args, rank, world, local_rank):
    import torch
    from mspms2_gb300 import build
    from mspms2_gb300.engine import TERMS_ALL, TERMS_LONG, TERMS_SHORT, Engine

    build.build()
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    system = make_system(args.workload)
    split_r = system.respa_split
    system.respa_split = 0.0  # the headline step is the full evaluation (reference split)
    n = system.natom
    stream = torch.cuda.current_stream()
    eng = Engine(system, precision=args.precision, device=local_rank)
    eng.set_stream(stream.cuda_stream)
    # launch geometry for this system (cell size, cluster size, k-force threads per site),
    # picked once before the warm-up, outside the timed region
    tuning = eng.autotune()
    pos = torch.tensor(np.stack([system.x, system.y, system.z]), dtype=torch.float64, device="cuda")
    fl = torch.empty((3, n), dtype=torch.float64, device="cuda")
    fs = torch.empty((3, n), dtype=torch.float64, device="cuda")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2
    ptrs = (pos[0].data_ptr(), pos[1].data_ptr(), pos[2].data_ptr())

    def step():
        return eng.compute_device(*ptrs, fl.data_ptr(), fs.data_ptr(), TERMS_ALL)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(local_rank)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    times = []
    for k in range(args.steps):
        flush.fill_(float(k))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step()
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    st = eng.stats()
    # the numerator both arms share: pairs inside the cutoff by FP64 distance (the engine's
    # own count, from FP32 distances, can differ by a few pairs at the cutoff shell)
    npairs = pairs_in_cutoff(system)
    ms_step = max_over_ranks(dist, statistics.mean(times), "cuda")
    value = job_rate(world, npairs, ms_step)

    launches = st["kernel_launches"]
    # per-stage device times: one more call with stage events on and the reciprocal-space
    # chain in line, so that each stage (and the roofline's kernel) is timed alone
    eng.set_kspace_overlap(False)
    eng.set_timing(True)
    flush.fill_(1.0)
    step()
    torch.cuda.synchronize()
    kms = eng.stats()["kernel_ms"]
    eng.set_timing(False)
    eng.set_kspace_overlap(True)

    # e2e through mg_compute with pinned host buffers
    hx = torch.from_numpy(np.ascontiguousarray(system.x)).pin_memory().numpy()
    hy = torch.from_numpy(np.ascontiguousarray(system.y)).pin_memory().numpy()
    hz = torch.from_numpy(np.ascontiguousarray(system.z)).pin_memory().numpy()
    hfl = torch.empty((3, n), dtype=torch.float64).pin_memory().numpy()
    hfs = torch.empty((3, n), dtype=torch.float64).pin_memory().numpy()
    for _ in range(2):
        eng.compute_into(hx, hy, hz, hfl, hfs)
    e2e_times = []
    for k in range(args.steps):
        flush.fill_(float(k))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.compute_into(hx, hy, hz, hfl, hfs)
        b.record(stream)
        b.synchronize()
        e2e_times.append(a.elapsed_time(b))
    e2e_ms = max_over_ranks(dist, statistics.mean(e2e_times), "cuda")
    e2e_value = job_rate(world, npairs, e2e_ms)

    extras = {}
    if not args.no_extras and rank == 0:
        # plain FP64 GPU path, same workload
        eng64 = Engine(system, precision="fp64", device=local_rank)
        eng64.set_stream(stream.cuda_stream)
        e64 = eng64.compute_device(*ptrs, fl.data_ptr(), fs.data_ptr(), TERMS_ALL)
        t64 = []
        for k in range(max(2, min(3, args.steps))):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            eng64.compute_device(*ptrs, fl.data_ptr(), fs.data_ptr(), TERMS_ALL)
            b.record(stream)
            b.synchronize()
            t64.append(a.elapsed_time(b))
        f64 = torch.cat([fl, fs]).clone()
        eng64.close()
        e32 = step()
        torch.cuda.synchronize()
        f32 = torch.cat([fl, fs])
        err = float(torch.linalg.vector_norm(f32 - f64) / torch.linalg.vector_norm(f64))
        ms64 = statistics.mean(t64)
        # each energy of the mixed path against the FP64 path, relative to the FP64 value and
        # to the sum of magnitudes of the terms the derived energies are made of; terms that
        # nearly vanish (the bonded ones at the template geometry) are judged against the
        # system's energy scale (the sum of magnitudes of all terms) instead
        elec_scale = sum(abs(e64[k]) for k in ("ureal", "ufourier", "uself", "uexcl", "uvacuum"))
        energy_scale = elec_scale + abs(e64["uvdw"]) + abs(e64["ushift"]) + abs(e64["uintra"])
        e_err = {}
        for k in ("uvdw", "ushift", "ureal", "uexcl", "ufourier", "uself", "uelec", "uinter", "virial_inter",
                  "ubond", "uangle", "uintra", "virial_intra"):
            d = abs(e32[k] - e64[k])
            ref = abs(e64[k])
            scale = elec_scale if k in ("uelec", "uinter", "virial_inter") else max(ref, 1e-6 * energy_scale)
            e_err[k] = {"rel": d / ref if ref > 0 else None, "rel_to_components": d / scale if scale > 0 else None,
                        "abs": d}
        extras["fp64_path"] = {"value": npairs / (ms64 * 1e-3), "ms_per_step": ms64,
                               "energy_err_mixed_vs_fp64": e_err,
                               "mixed_over_fp64": ms64 / ms_step, "rms_rel_force_err_mixed_vs_fp64": err}
        # device-resident NVT Nose-Hoover RESPA (mg_md_run, the reference's vver_nh_3):
        # inner steps of 0.5 fs with bonded + pairs inside 7 A, outer 2 fs step with the
        # 7-10 A shell and reciprocal space; Verlet skin 1 A
        if split_r > 0:
            extras["respa"] = md_extras(system, split_r, args.precision, local_rank)
        extras["hmc_batch"] = hmc_extras(local_rank)
        extras["siman_batch"] = siman_batch_extras(local_rank)
        extras["derivatives"] = adjoint_extras(system, args.precision, local_rank)
        extras["force_matching"] = force_matching_extras(local_rank)
        extras["c5_butane_tubes"] = c5_extras(local_rank)
        extras["c1_nvt"] = c1_extras(local_rank)
        if not args.no_cpu_baseline:
            threads = host_threads()
            cpu = cpu_baseline(system, threads)
            extras["cpu_baseline"] = {"value": npairs / cpu["t_step_s"], "unit": "pair-interactions/s",
                                      "cores": threads, "kind": "port", "sample": cpu["sample"],
                                      "t_step_s": cpu["t_step_s"], "t_frclong_s": cpu["t_frclong_s"],
                                      "t_frcshort_s": cpu["t_frcshort_s"], "host_cores": os.cpu_count()}

    # roofline of the dominant stage (FP32 pipe: no stage is a dense contraction)
    kvec = st["kvectors"]
    nrows, nkz = ewald_rows(tuple(system.kmax), system.ksqmax) if kvec else (0, 0)
    stages = {"pair": (kms[1], FLOP_PAIR * npairs), "kspace_sk": (kms[3], FLOP_K_S * kvec * n),
              "kspace_force": (kms[4], FLOP_K_F * kvec * n)}
    executed = {"pair": FLOP_PAIR * npairs, "kspace_sk": (FLOP_SK_ROWKZ * nkz + FLOP_SK_ROW * nrows) * n,
                "kspace_force": (FLOP_KF_ROWKZ * nkz + FLOP_KF_ROW * nrows) * n}
    dom = max(stages, key=lambda k: stages[k][0])
    t_ms, flops = stages[dom]
    sm_count, sm_mhz, peak_basis = fp32_peak_inputs(local_rank, clk)
    peak = sm_count * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    achieved = flops / (t_ms * 1e-3) / 1e12 if t_ms > 0 else 0.0
    # DRAM bytes per launch of that kernel from the committed ncu summary of this workload
    traffic = None
    kf_tensor = bool(kvec) and args.precision == "mixed" and system.kmax[2] <= 30
    kernel_of = {"pair": "k_pair", "kspace_sk": "k_sk_mma",
                 "kspace_force": "k_kforce_mma" if kf_tensor else "k_kforce_mm"}
    tf = os.path.join(ROOT, "profiles", f"kernels_{args.workload}.md")
    if os.path.exists(tf):
        for ln in open(tf):
            parts = ln.split()
            if len(parts) == 4 and parts[0] == "traffic_bytes_per_launch" and parts[1] == kernel_of[dom]:
                traffic = float(parts[3])
    # per-stage figures of the pair and list kernels: the pair stage by the work model (55 FLOP
    # per pair, counted once) and as neighbour streaming against HBM (per listed entry 4 B index
    # + 16 B shift, per j-cluster of the half list its 8 slots x 32 B, per site 16 B position and
    # 24 B force), the list stage by the bytes it writes and reads (per entry 4 B index, 16 B
    # shift, 4 B image; per site its FP64 position and wrapped position)
    hbm = measured_peaks().get("hbm_gbs")
    nent = st["cluster_pairs"]
    pair_bytes = neighbour_streaming_bytes(nent, n)
    list_bytes = list_build_bytes(nent, n)
    stage_roofline = {
        "pair": {"ms": kms[1], "tflops_work_model": FLOP_PAIR * npairs / (kms[1] * 1e-3) / 1e12 if kms[1] else None,
                 "frac_fp32": FLOP_PAIR * npairs / (kms[1] * 1e-3) / 1e12 / peak if kms[1] else None,
                 "neighbour_streaming_gbs": pair_bytes / (kms[1] * 1e-3) / 1e9 if kms[1] else None,
                 "hbm_frac": pair_bytes / (kms[1] * 1e-3) / 1e9 / hbm if (kms[1] and hbm) else None,
                 "bytes_per_call": pair_bytes},
        "list": {"ms": kms[0], "gbs": list_bytes / (kms[0] * 1e-3) / 1e9 if kms[0] else None,
                 "hbm_frac": list_bytes / (kms[0] * 1e-3) / 1e9 / hbm if (kms[0] and hbm) else None,
                 "bytes_per_call": list_bytes},
        "peak_basis": "FP32 as in roofline; HBM of measured (MEASURED_PEAKS.json hbm_gbs); the list and "
                      "packed operands mostly stay in the 129 MB L2, so these rates exceed what DRAM moves"}
    if rank != 0:
        return 0
    line = {"metric": "pair_interactions_per_s", "value": value, "unit": "pair-interactions/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair math / f64 accumulation"
            if args.precision == "mixed" else "f64", "data": "synthetic (seeded lattice water)",
            "config": {"workload": args.workload, "sites": n, "molecules": system.nmole, "box_A": float(system.box[0]),
                       "rc_A": system.rcutoff, "ewald_alpha": system.kappa, "kmax": list(system.kmax),
                       "ksqmax": system.ksqmax, "kvectors_half_space": kvec, "kspace_rows": nrows,
                       "kspace_row_kz": nkz, "pairs_in_cutoff": npairs,
                       "pairs_in_cutoff_engine_fp32": st["pairs_within_cutoff"],
                       "l2": "256 MiB flush before every step; steps timed one by one with CUDA events",
                       "parallelism": f"replicas x{world}",
                       "tuning": {k: tuning[k] for k in ("cell_scale", "zcap_scale", "kforce_threads", "ms_default",
                                                          "ms_tuned")}},
            "e2e": {"value": e2e_value, "unit": "pair-interactions/s", "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": 3 * 8 * n, "d2h_bytes_per_step": 6 * 8 * n + 8 * 18},
            "gpu_launches": launches * args.steps,
            "stage_ms": {"list": kms[0], "pair": kms[1], "intra_bonded": kms[2], "kspace_sk": kms[3],
                         "kspace_force": kms[4], "solid_fluid": kms[5], "reduce": kms[6], "total": kms[7],
                         "note": "stages timed alone (reciprocal space in line); the timed steps run the "
                                 "reciprocal-space chain on a second stream beside the list and pairs"},
            "roofline": {"bound": "fp32", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "executed_tflops": executed[dom] / (t_ms * 1e-3) / 1e12 if t_ms > 0 else 0.0,
                         "executed_note": "FLOP the kernel's algorithm executes (the table passes do fewer than "
                                          "the work model counts per k-vector)",
                         "peak_basis": peak_basis},
            "clocks": clk, "stage_roofline": stage_roofline}
    if kf_tensor:
        tf = kf_tensor_flops(tuple(system.kmax), system.ksqmax, n)
        f16_peak = measured_peaks().get("bf16_tflops") or 1900.0
        line["kspace_force_tensor"] = {
            "kernel": "k_kforce_mma", "ms": kms[4], "mma_tflop": tf / 1e12, "operands": "FP16 hi + lo, kind::f16",
            "achieved_tflops": tf / (kms[4] * 1e-3) / 1e12 if kms[4] > 0 else 0.0, "peak_tflops": f16_peak,
            "frac": tf / (kms[4] * 1e-3) / 1e12 / f16_peak if kms[4] > 0 else 0.0,
            "peak_basis": "of measured: MEASURED_PEAKS.json bf16_tflops (cuBLAS bf16 burst; FP16 and BF16 MMAs run at "
                          "one rate)" if measured_peaks().get("bf16_tflops") else "of fallback (1.9 PFLOP/s bf16)"}
    if kvec and args.precision == "mixed" and system.kmax[2] <= 30:
        tf = sk_tensor_flops(tuple(system.kmax), system.ksqmax, n)
        f16_peak = measured_peaks().get("bf16_tflops") or 1900.0
        line["kspace_sk_tensor"] = {
            "kernel": "k_sk_mma", "ms": kms[3], "mma_tflop": tf / 1e12, "operands": "FP16 hi + lo, kind::f16",
            "achieved_tflops": tf / (kms[3] * 1e-3) / 1e12 if kms[3] > 0 else 0.0, "peak_tflops": f16_peak,
            "frac": tf / (kms[3] * 1e-3) / 1e12 / f16_peak if kms[3] > 0 else 0.0,
            "peak_basis": "of measured: MEASURED_PEAKS.json bf16_tflops (cuBLAS bf16 burst; FP16 and BF16 MMAs run at "
                          "one rate)" if measured_peaks().get("bf16_tflops") else "of fallback (1.9 PFLOP/s bf16)",
            "note": "structure factors as FP16 MMAs (3-term split product, FP32 accumulation in tensor memory); "
                    "FLOP issued, padding included; the stage time includes operand generation on the CUDA cores"}
    if "cpu_baseline" in extras:
        line["cpu_baseline"] = extras.pop("cpu_baseline")
    line.update(extras)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)
    if args.md_dt_sweep:
        from mspms2_gb300 import build
        build.build()
        if rank == 0:
            print(json.dumps(md_dt_sweep(args.precision, local_rank)), flush=True)
        return 0
    if args.nve_drift:
        from mspms2_gb300 import build
        build.build()
        if rank == 0:
            print(json.dumps(nve_drift(local_rank)), flush=True)
        return 0
    if args.nve_drift_scan:
        from mspms2_gb300 import build
        build.build()
        if rank == 0:
            print(json.dumps(nve_drift_scan(local_rank)), flush=True)
        return 0
    return run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
