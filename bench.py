"""Benchmark: GLL-point x azimuth updates/s of the AxiSEM3D time step on GB300.

Workload (default): the element-level stiffness batching benchmark -- 200,000
independent solid elements, nPol = 4, spherical geometry in the mantle, Nu_e
log-uniform in [8, 256] (nr = 2 Nu + 1), transversely isotropic moduli perturbed +-5 %
per GLL point and azimuthal sample (physical-space path), 3 SLS with Q_mu in [80, 600]
(CG4), complex FP32 displacement ~ N(0,1) alpha^-1.5.  One step = Newmark update +
element stiffness + assembly (Newmark::solve's loop body).  Inputs are seeded synthetic
data resident in HBM; the working set (~70 GB) is far larger than L2, so no flush is
needed between steps.

value  = sum_e 25 nr_e x steps / device time (CUDA events on the library's stream).
e2e    = the same through the C-ABI with host buffers: each step copies the
         displacement in from pinned host memory, steps, and copies it back, the copies
         streamed (ax3d_set_field_async / ax3d_get_field_async) so that they overlap the
         steps; the synchronous form is reported beside it.
Reference arm (--impl reference): the CPU port of the same loop (the oracle's arithmetic
with O(nr log nr) FP32 transforms, as the reference uses FFTW), one process per host
core over a static element partition, on a bounded sample.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GLL-pt*azimuth updates/s (element-local count), fused stiffness+Newmark step"
UNIT = "updates/s"


def run_earth3d(args, world, rank, local, full_steps=20000):
    """3-D Earth full solver: the layered half disk refined to ~63,000 quads (about 10 s
    shortest period), seeded Gaussian-random dlnVs / dlnVp (4 % RMS, 500 km lateral, 200 km
    radial correlation) forcing physical-space stiffness everywhere in the solid, Nu fixed
    at 256, fluid outer core with solid-fluid coupling, compensated Newmark, 200 stations.
    The run covers 20,000 steps; here a window of max(steps, 50) steps is timed and the
    time-to-seismogram of the whole run is the pre-loop plus 20,000 times the step time.
    0.8 of the mesh's CFL step (the step 3-D runs at the top orders are stable at)."""
    import tempfile
    import torch
    from axisem3d_gb300 import build, solver
    from axisem3d_gb300.capi import Ax3dDomain
    from axisem3d_gb300.nu_learn import DT_FACTOR, model_strings
    build.build()
    window = max(args.steps, 50)
    d = Path(tempfile.mkdtemp()) / "input"
    mesh = dict(n_theta=320, h_mantle=30e3, h_core=33e3)
    solver.write_inputs(d, mesh_kw=mesh, steps=full_steps, hdur=10.0, n_stations=200, seed=args.seed, nu=256,
                        models3d=model_strings(1000 + args.seed))
    p = d / "inparam.time_src_recv"
    p.write_text(p.read_text().replace("TIME_DELTA_T_FACTOR 1.0", f"TIME_DELTA_T_FACTOR {DT_FACTOR}"))
    t0 = time.perf_counter()
    sim = solver.Simulation(d)
    spec = sim.build(kahan=True, preloop="gpu")
    t_pre = time.perf_counter() - t0
    upd = int(spec.p_nr.astype(np.int64).sum())
    dom = Ax3dDomain(spec, device=local)
    tune = dom.autotune(2)
    dom.enable_timers(True)
    dom.step(args.warmup)
    dom.read_timers()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dom.step(window)
    seis = dom.seismograms(0, args.warmup + window)
    wall = time.perf_counter() - t0
    tm = dom.read_timers()
    dom.close()
    dev_s = tm["step"][0] / 1e3
    if rank != 0:
        return
    line = {"metric": "GLL-pt*azimuth updates/s (unique-point count), 3-D full solver", "value": upd * window / dev_s,
            "unit": UNIT, "n_gpus": world, "steps": window, "warmup": args.warmup,
            "ms_per_step": dev_s * 1e3 / window, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": f"3-D Earth full solver, {spec.n_elements} quads, Nu=256, Gaussian-random 3-D "
                                   f"model, fluid core, compensated Newmark, {len(spec.r_elem)} stations",
                       "points": spec.n_points, "dt": spec.dt, "schedule": tune[:120]},
            "phases_ms_per_step": {k: v[0] / window for k, v in tm.items()},
            "gpu_launches": sum(v[1] for k, v in tm.items() if k != "step"),
            "preloop_s": t_pre, "wall_ms_per_step": wall * 1e3 / window,
            "time_to_seismogram_s": {"run_steps": full_steps, "estimate": t_pre + full_steps * dev_s / window},
            "finite": bool(np.isfinite(seis).all())}
    print(json.dumps(line), flush=True)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--elements", type=int, default=200_000)
    ap.add_argument("--att", default="cg4", choices=["cg4", "full", "none"])
    ap.add_argument("--material", default="3d", choices=["3d", "1d"],
                    help="3d: moduli per azimuth sample (physical-space path, default); 1d: per GLL point "
                         "(Fourier-space path)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--schedule", default="",
                    help="ratio,policy,nside,merge: pin the element bucket schedule instead of autotuning it")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=0, help="elements per CPU worker (0 = auto)")
    ap.add_argument("--workload", default="elements", choices=["elements", "halfdisk", "earth3d", "ensemble"],
                    help="elements: the element-level benchmark (default); halfdisk: the full solver; earth3d: "
                         "the 3-D full solver at Nu 256; ensemble: the batched ensemble")
    return ap.parse_args()


MATERIAL = {"3d": "3-D (physical-space) material", "1d": "1-D (Fourier-space) material"}


def att_kind(name):
    from axisem3d_gb300.spec import ATT_CG4, ATT_FULL, ATT_NONE
    return {"cg4": ATT_CG4, "full": ATT_FULL, "none": ATT_NONE}[name]


def algorithmic_bytes(spec, att, in3d=True):
    """Compulsory HBM bytes of one element-stiffness pass (each array read/written once).

    Per element with n = Nu+1 orders and nr samples: displacement in 600 n, element force
    out 600 n, geometry 500 B, theta tables 400 B; 3-D (physical space): TI moduli
    5*25*4*nr, SLS state (nsls+1)*nr*6*npa*4 read + write, attenuation moduli 2*nr*npa*4
    (npa = 4 CG4 / 25); 1-D (Fourier space): TI moduli 5*25*4, complex SLS state
    (nsls+1)*n*6*npa*8 read + write, attenuation moduli 2*npa*4."""
    nr = spec.element_nr().astype(np.int64)
    n = nr // 2 + 1
    rows = nr if in3d else 1
    b = 600 * n + 600 * n + 500 + 400 + 5 * 25 * 4 * rows
    if att != "none":
        npa = 4 if att == "cg4" else 25
        state = nr * 6 * npa * 4 if in3d else n * 6 * npa * 8
        b = b + 2 * (spec.nsls + 1) * state + 2 * rows * npa * 4
    return int(b.sum())


def point_bytes(spec):
    """Newmark update + assembly per step: stiff, u, v, a read and written, element
    force read once, 1/M per point (row kernels)."""
    ns, _ = spec.field_sizes()
    return int(8 * ns * (4 + 4) + 8 * ns * 2 + 4 * spec.n_points)


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = [r.split(",") for r in getattr(self, "out", "").strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, x):
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(x)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return x


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per algorithmic byte of the
# element pass, measured by ncu over every element launch of one step of the
# 20,000-element case of this workload (same distributions, ~5.5 GB of element data, far
# above L2).  The 200,000-element workload is too large to capture with more than one ncu
# pass; its traffic grows in proportion to the elements processed, so it is this ratio
# times its algorithmic bytes.  Re-measured whenever the element kernel or the schedule
# changes (this figure: schedule policy 3 with merged launches, the autotuner's pick).
TRAFFIC_PER_ALGO_BYTE = 1.034


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------------ CPU (oracle) arm
# The CPU baseline is the oracle's loop (the reference's per-element arithmetic) built with
# O(nr log nr) FP32 transforms in place of the checker's exact DFT, as the reference runs
# FFTW plans (oracle/ax3d_fft.hpp): kind "port", variant "port-fft".  One process per host core, each on its
# own partition of elements drawn from the workload's distributions (one MPI rank per core
# in the reference).
def _cpu_worker(a):
    """Build one partition sample and time the CPU baseline's loop body on it."""
    seed, n_elem, att, steps, in3d = a
    sys.path.insert(0, str(ROOT))
    from axisem3d_gb300 import workloads as W
    from oracle.oracle_py import OracleDomain
    spec = W.element_benchmark(n_elem=n_elem, seed=seed, att=att_kind(att), in3d=in3d)
    d = OracleDomain(spec, fft=True)
    d.set("displ", "solid", W.benchmark_displacement(spec, seed=seed + 1).astype(np.complex128))
    d.step(1)  # first touch, transform plans
    t0 = time.perf_counter()
    d.step(steps)
    dt = time.perf_counter() - t0
    return W.updates_per_step(spec) * steps, dt, spec.element_nr().tolist()


def nr_histogram(nr):
    """Quartiles and mean of the sample's ring sizes, for the record."""
    q = np.percentile(np.asarray(nr), [0, 25, 50, 75, 100])
    return f"nr mean {float(np.mean(nr)):.1f}, quartiles {'/'.join(str(int(x)) for x in q)}"


def cpu_baseline(att, cores, sample, steps=2, seed=1000, in3d=True):
    import multiprocessing as mp
    from oracle.oracle_py import build_oracle
    build_oracle()
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(seed + 7 * i, sample, att, steps, in3d) for i in range(cores)])
    upd = sum(r[0] for r in res)
    wall = max(r[1] for r in res)
    nrs = [x for r in res for x in r[2]]
    return upd / wall, dict(cores=cores, sample=f"FFT port: {cores} partitions x {sample} elements x {steps} step(s) of the "
                            f"same Nu / material distributions (seeds {seed}..; {nr_histogram(nrs)}; the 200,000-"
                            f"element workload: nr mean ~144)", wall_s=wall)


CPU_SAMPLE = 160  # elements per core: ~10-30 s of CPU work per call


def run_reference(args, world, rank):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    sample = args.cpu_sample or CPU_SAMPLE
    vals = []
    for _ in range(max(1, min(args.steps, 3))):
        v, info = cpu_baseline(args.att, cores, sample, in3d=args.material == "3d")
        vals.append(v)
    v = float(np.median(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": f"element stiffness batching, {args.elements} TI elements, Nu 8-256 "
                                   f"log-uniform, 3 SLS {args.att}, {MATERIAL[args.material]}"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": info["cores"], "kind": "port",
                             "variant": "port-fft", "sample": info["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference (C++/Eigen/FFTW/MPI) does not build here; the CPU port of the same loop "
                    "with O(nr log nr) FP32 transforms is timed, one process per core"}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GB300 arm
def run_gb300(args, world, rank, local):
    from axisem3d_gb300 import build
    from axisem3d_gb300 import workloads as W
    from axisem3d_gb300.capi import Ax3dDomain
    build.build()
    t_build = time.perf_counter()
    in3d = args.material == "3d"
    spec = W.element_benchmark(n_elem=args.elements, seed=args.seed + rank, att=att_kind(args.att), in3d=in3d)
    u0 = W.benchmark_displacement(spec, seed=args.seed + 100 + rank)
    dom = Ax3dDomain(spec, device=local)
    dom.set("displ", "solid", u0)
    if args.schedule:
        r, pol, ns, mg = args.schedule.split(",")
        dom.set_schedule(float(r), int(pol), int(ns), bool(int(mg)))
        tune = f"pinned {args.schedule}"
    else:
        tune = dom.autotune(2)  # the bucket schedule from timed element passes on this domain
    t_build = time.perf_counter() - t_build
    upd = W.updates_per_step(spec)

    dom.enable_timers(True)
    dom.step(args.warmup)
    dom.read_timers()
    barrier(world)
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        dom.step(args.steps)
        wall = time.perf_counter() - t0
    tm = dom.read_timers()
    dev_s = tm["step"][0] / 1e3
    dev_s_max = allmax(world, dev_s)
    barrier(world)

    # e2e through the C-ABI with pinned host buffers: every step copies its displacement in
    # and its result out.  Measured twice: synchronous calls (copy in, step, copy out in
    # turn) and streamed (ax3d_set_field_async / ax3d_get_field_async: the next input is
    # copied in and the last result copied out while a step runs); the streamed figure is
    # the headline.
    e2e = None
    if not args.no_e2e:
        import torch
        n = dom.nsolid
        dom.enable_timers(False)
        # one pinned buffer each way (8 B x field size each): every step's input is the same
        # state, and the result copies are ordered on one copy stream
        pin_in = torch.empty(n, dtype=torch.complex64, pin_memory=True).numpy()
        pin_out = torch.empty(n, dtype=torch.complex64, pin_memory=True).numpy()
        pin_in[:] = dom.get("displ")
        ke = max(3, args.steps)  # the streamed loop fills and drains once: time as many steps as `value`
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(ke):
            dom.set("displ", "solid", pin_in)
            dom.step(1)
            dom.get("displ", "solid", out=pin_out)
        sync_s = allmax(world, (time.perf_counter() - t0) / ke)
        barrier(world)
        t0 = time.perf_counter()
        dom.set_async("displ", "solid", pin_in)
        for k in range(ke):
            if k + 1 < ke:
                dom.set_async("displ", "solid", pin_in)
            dom.step(1)
            dom.get_async("displ", "solid", pin_out)
        dom.sync_fields()
        e2e_s = allmax(world, (time.perf_counter() - t0) / ke)
        e2e = {"value": upd * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(8 * n),
               "d2h_bytes_per_step": int(8 * n), "ms_per_step": e2e_s * 1e3,
               "transfer": "streamed: double-buffered async copies overlapping the steps",
               "sync_ms_per_step": sync_s * 1e3, "sync_value": upd * world / sync_s}

    if rank != 0:
        return
    elem_ms = tm["elements"][0] / args.steps
    abytes = algorithmic_bytes(spec, args.att, in3d)
    peak, src = peaks()
    achieved = abytes / (elem_ms / 1e3) / 1e9
    launches = sum(v[1] for k, v in tm.items() if k != "step")
    cpu = None
    if not args.no_cpu_baseline:
        try:
            v, info = cpu_baseline(args.att, os.cpu_count() or 1, args.cpu_sample or CPU_SAMPLE, in3d=in3d)
            cpu = {"value": v, "unit": UNIT, "cores": info["cores"], "kind": "port", "variant": "port-fft",
                   "sample": info["sample"]}
        except Exception as e:  # the CPU leg must not hide the GPU number
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "variant": "port-fft",
                   "sample": f"failed: {e}"}
    line = {
        "metric": METRIC, "value": upd * args.steps * world / dev_s_max, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_s_max * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": f"element stiffness batching, {args.elements} TI elements, Nu 8-256 "
                               f"log-uniform (nr = 2Nu+1), 3 SLS {args.att}, {MATERIAL[args.material]}, "
                               f"fused stiffness+Newmark step", "elements": args.elements,
                   "updates_per_step": upd, "parallelism": f"replicas x{world}", "schedule": tune[:80],
                   "l2": "working set > L2 (no flush needed)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": (TRAFFIC_PER_ALGO_BYTE * abytes if in3d and args.att == "cg4" else None),
                     "traffic_unit": "bytes per step (ncu DRAM bytes per algorithmic byte x algorithmic bytes)",
                     "peak_source": src,
                     "kernel": ("element stiffness (k_elem_phys, all buckets)" if in3d
                                else "element stiffness (k_elem_fourier_solid)"),
                     "algorithmic_bytes_per_step": abytes, "kernel_ms_per_step": elem_ms},
        "phases_ms_per_step": {k: v[0] / args.steps for k, v in tm.items()},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "e2e": e2e,
        "cpu_baseline": cpu,
        "host_wall_ms_per_step": wall * 1e3 / args.steps,
        "setup_s": t_build,
    }
    print(json.dumps(line), flush=True)


def run_halfdisk(args, world, rank, local):
    """Full solver on the seeded half-disk mesh (~6,000 quads, Nu = 2, fluid core, 2,000
    steps, 20 stations): unique-point updates/s and time-to-seismogram (host inputs in, NetCDF
    seismograms out), with the CPU oracle on the same mesh for a bounded window of steps."""
    import tempfile
    from axisem3d_gb300 import build, solver
    from axisem3d_gb300.capi import Ax3dDomain
    build.build()
    d = Path(tempfile.mkdtemp()) / "input"
    solver.write_inputs(d, steps=2000, hdur=50.0, n_stations=20, seed=args.seed)
    sim = solver.Simulation(d)
    spec = sim.build()
    upd = int(spec.p_nr.astype(np.int64).sum())  # sum_p nr_p per step
    dom = Ax3dDomain(spec, device=local)
    dom.enable_timers(True)
    dom.step(args.warmup)
    dom.reset()
    dom.read_timers()
    t0 = time.perf_counter()
    rtz, _ = sim.run(domain=dom)
    sim.write_netcdf(rtz)
    tts = time.perf_counter() - t0
    tm = dom.read_timers()
    dev_s = tm["step"][0] / 1e3
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        from oracle.oracle_py import OracleDomain
        o = OracleDomain(spec)
        ncpu = 100
        tc = time.perf_counter()
        o.step(ncpu)
        tc = time.perf_counter() - tc
        cpu = {"value": upd * ncpu / tc, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{ncpu} steps of the same mesh, one process"}
    line = {"metric": "GLL-pt*azimuth updates/s (unique-point count), full solver", "value": upd * sim.nsteps / dev_s,
            "unit": UNIT, "n_gpus": world, "steps": sim.nsteps, "warmup": args.warmup,
            "ms_per_step": dev_s * 1e3 / sim.nsteps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": f"half-disk full solver, {spec.n_elements} quads, Nu=2, fluid core, "
                                   f"{sim.nsteps} steps, {len(spec.r_elem)} stations", "points": spec.n_points},
            "time_to_seismogram_s": tts, "phases_ms_per_step": {k: v[0] / sim.nsteps for k, v in tm.items()},
            "gpu_launches": sum(v[1] for k, v in tm.items() if k != "step"), "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def run_ensemble(args, world, rank, local, members=32, steps=200):
    """Batched ensemble in the form of the ensemble configuration, scaled to this mesher: 32
    independent 3-D Earths (seeded Gaussian-random dlnVs / dlnVp, 4 % RMS), meshes of 48 to 96
    elements in colatitude (about 2,700 to 5,900 quads), per-element Nu log-uniform in 4-256
    (the range a learned Nu field spans), moment-tensor sources at 10-600 km depth,
    compensated Newmark, 0.8 of the mesh's CFL step (the step the 3-D runs are stable at).
    All members run in one domain whose step is one captured CUDA graph with an autotuned
    bucket schedule, against (1) the same members run one after another, each in its own
    domain, and (2) the plain full-Nu solver (Nu = 256 everywhere) on the same members one
    after another.  A fixed window of `steps` steps (the configuration's 10,000 scale
    linearly); pre-loops on the GPU, timed apart and added for time-to-seismogram."""
    import tempfile
    import torch
    from axisem3d_gb300 import build, ensemble, solver
    from axisem3d_gb300.capi import Ax3dDomain
    from axisem3d_gb300.nu_learn import DT_FACTOR, model_strings
    build.build()
    rng = np.random.default_rng(args.seed)
    specs, sims = [], []
    pre_var = []
    for i in range(members):
        d = Path(tempfile.mkdtemp()) / "input"
        nt = int(rng.choice([48, 64, 96]))
        solver.write_inputs(d, mesh_kw=dict(n_theta=nt), steps=steps, hdur=50.0, n_stations=10, seed=args.seed + i,
                            depth_km=float(rng.uniform(10, 600)), nu=256, models3d=model_strings(100 + i))
        p = d / "inparam.time_src_recv"
        p.write_text(p.read_text().replace("TIME_DELTA_T_FACTOR 1.0", f"TIME_DELTA_T_FACTOR {DT_FACTOR}"))
        sim = solver.Simulation(d)
        sim.build(preloop="gpu")  # mesh and element count
        nu_e = np.round(np.exp(rng.uniform(np.log(4), np.log(256), len(sim.e_pts)))).astype(np.int64)
        t0 = time.perf_counter()
        specs.append(sim.build(kahan=True, nu_elem=nu_e, preloop="gpu"))
        pre_var.append(time.perf_counter() - t0)
        sims.append(sim)
    dt = min(s.dt for s in specs)
    for s in specs:
        s.dt = dt
        s.stf = specs[0].stf
    spec, info = ensemble.concat(specs)
    upd = int(spec.p_nr.astype(np.int64).sum())
    dom = Ax3dDomain(spec, device=local)
    tune = dom.autotune(2)
    dom.step(args.warmup)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dom.step(steps)
    seis = dom.seismograms(0, args.warmup + steps)
    t_batch = time.perf_counter() - t0
    dom.close()

    def sequential(member_specs):
        t = 0.0
        ok = True
        for s in member_specs:
            d1 = Ax3dDomain(s, device=local)
            d1.autotune(2)
            d1.step(args.warmup)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            d1.step(steps)
            ok &= bool(np.isfinite(d1.seismograms(0, args.warmup + steps)).all())
            t += time.perf_counter() - t0
            d1.close()
        return t, ok

    t_seq, _ = sequential(specs)
    # the plain full-Nu solver on the same members (pre-loop timed, then the loop)
    pre_full, full_specs = [], []
    for sim in sims:
        t0 = time.perf_counter()
        fs = sim.build(kahan=True, preloop="gpu")
        pre_full.append(time.perf_counter() - t0)
        fs.dt = dt
        fs.stf = specs[0].stf
        full_specs.append(fs)
    upd_full = int(sum(int(fs.p_nr.astype(np.int64).sum()) for fs in full_specs))
    t_full, ok_full = sequential(full_specs)
    if rank != 0:
        return
    tts_batched = sum(pre_var) + t_batch
    tts_full = sum(pre_full) + t_full
    line = {"metric": "GLL-pt*azimuth updates/s (unique-point count), batched ensemble", "value": upd * steps / t_batch,
            "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": args.warmup,
            "ms_per_step": t_batch * 1e3 / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": f"ensemble of {members} 3-D half-disk Earths in one domain (CUDA graph per step, "
                                   "autotuned buckets), per-element Nu 4-256, compensated Newmark",
                       "elements": spec.n_elements, "points": spec.n_points, "autotune": tune[:200]},
            "sequential_value": upd * steps / t_seq, "batched_over_sequential": t_seq / t_batch,
            "full_nu": {"updates_per_step": upd_full, "loop_s": t_full, "preloop_s": sum(pre_full),
                        "loop_over_batched": t_full / t_batch, "finite": ok_full},
            "time_to_seismogram": {"batched_s": tts_batched, "sequential_full_nu_s": tts_full,
                                   "ratio": tts_full / tts_batched, "preloop_batched_s": sum(pre_var)},
            "finite": bool(np.isfinite(seis).all())}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "halfdisk":
        run_halfdisk(args, world, rank, local)
    elif args.workload == "earth3d":
        run_earth3d(args, world, rank, local)
    elif args.workload == "ensemble":
        run_ensemble(args, world, rank, local)
    else:
        run_gb300(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
