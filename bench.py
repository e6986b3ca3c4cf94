"""Throughput benchmark of the ensemble-trajectory path on GB300.

Workload (the configuration the headline metric is quoted on): SAE argon
(Tong-Lin preset, Ip = 15.76 eV), Cos2 laser 800 nm, 1.2e14 W/cm^2, 2 cycles,
circular polarization; SFA-SPANE Monte-Carlo sampling of 1e7 electrons
(1e4 time samples uniform over the pulse x 1e3 transverse momenta uniform in
[-1, 1] a.u.); SCTS phase; integration to t_final = pulse end + 2 cycles with
rtol 1e-6; coherent 1000 x 1000 momentum grid spanning +-2 a.u.

A step is one whole job: sampling, integration, collection and the
deterministic deposit.  `value` is effective trajectories per second of the
FP32-bulk path with all buffers resident on the device; `e2e` is the same
metric through etraj_run with host output buffers (spectrum copied back every
step).  The FP64 plain path is run on the same job for the speed ratio and
the PMD error (relative L2 of |A|^2 against the FP64 result).

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun each rank runs its own Monte-Carlo shard (seed = rank):
weak scaling, no data-path collective.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import __graft_entry__  # noqa: E402

et = __graft_entry__.load_package()
from etraj_gb300 import abi  # noqa: E402

METRIC = "trajectories/sec on 1 GB300 (FP32-bulk vs FP64 plain, PMD L2 <=1e-3); p50/p99 job latency"
UNIT = "trajectories/s"
WORKLOAD = ("SAE Ar, Cos2 800 nm 1.2e14 W/cm^2 2 cyc CP, SPANE Monte-Carlo 1e4 t x 1e3 kd, "
            "SCTS, t_final = pulse end + 2 cycles, rtol 1e-6, coherent 1000x1000 PMD +-2 a.u.")


def make_job(precision="fp32_bulk", seed=0, t_num=10000, kt_num=1000):
    laser = et.Cos2Laser(peak_int=1.2e14, wave_len=800.0, cyc_num=2, ellip=1.0)
    T = laser.Period()
    half = laser.CycNum() * T / 2  # the Cos2 envelope spans [-N T/2, N T/2]
    return et.make_job(init_cond_method="SPANE", laser=laser, target=et.get_atom("Ar"), dimension=2,
                       sample_t_intv=(-half, half), sample_t_num=t_num, traj_t_final=half + 2 * T,
                       final_p_max=(2.0, 2.0), final_p_num=(1000, 1000), sample_monte_carlo=True,
                       mc_kt_num=kt_num, mc_kd_max=1.0, traj_phase_method="SCTS", seed=seed,
                       precision=precision)


# FP32 operations of one Tsit5 step of the bulk integrator for 2D SAE SCTS, counted
# from integrate_fp32.cu (an FMA counts 2, every other arithmetic instruction 1,
# MUFU ops 1): right-hand side 52 (field 12, radius and rsqrt 14, three exponentials
# 6, bracket and force 12, phase 8) x 6 stages = 312; stage combinations
# 2*(1+2+3+4+5+6)*5 = 210; error estimate 5*(2*7+6) = 100; compensated update
# 5*8 = 40; clock, controller and bookkeeping ~40.  Total 702 per step attempt.
FLOPS_PER_STEP_SAE_2D_SCTS = 702


def rank_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                mx = float(p[1])
            except ValueError:
                continue
            for name, v in zip(names, p[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def cpu_baseline(job_fn, seconds_target=15.0):
    """Times the CPU oracle (the reference's algorithm restated in C, OpenMP over time
    samples) on a bounded sample of the workload: a slice of the time samples."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle  # the checker doubles as the timed CPU port

    sys.path.pop(0)
    cores = _oracle.nthreads()
    t_num = 40
    while True:
        job = job_fn(t_num)
        t0 = time.perf_counter()
        _, _, sc = _oracle.run(job)
        dt = time.perf_counter() - t0
        if dt > seconds_target / 4 or t_num >= 10000:
            break
        t_num = min(10000, int(t_num * max(2.0, seconds_target / 3 / max(dt, 1e-3))))
    return {"value": sc["num_effective"] / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d of 10000 time samples x 1000 kd (%d effective trajectories, %.1f s)"
                      % (t_num, int(sc["num_effective"]), dt)}


def run_reference(args):
    rank, world, _ = rank_env()
    if rank != 0:
        return 0
    job_fn = lambda n: make_job("fp64", seed=0, t_num=n)  # noqa: E731
    base = cpu_baseline(job_fn, seconds_target=12.0)
    n = int(base["sample"].split(" ")[0])
    times, effs = [], []
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle

    sys.path.pop(0)
    for i in range(args.warmup + args.steps):
        job = make_job("fp64", seed=i, t_num=n)
        t0 = time.perf_counter()
        _, _, sc = _oracle.run(job)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
            effs.append(sc["num_effective"])
    value = sum(effs) / sum(times)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "sample": base["sample"]},
            "cpu_baseline": dict(base, value=value),
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference = the C restatement of eTraj.jl's algorithm on the host cores "
                    "(Julia is not installed on this machine)"}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--t-num", type=int, default=10000,
                    help="time samples (x 1000 kd candidates); 10000 is the full workload")
    ap.add_argument("--precision", default="fp32_bulk", choices=["fp32_bulk", "fp64"],
                    help="path timed as `value` (fp64 profiles the plain kernel)")
    ap.add_argument("--no-fp64-compare", action="store_true",
                    help="skip the FP64 run used for the speed ratio and PMD error (profiling)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import torch.distributed as dist

    rank, world, local = rank_env()
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    eng = et.Engine(device=local)
    stream = torch.cuda.Stream(device=dev)
    eng.set_stream(stream.cuda_stream)

    job = make_job(args.precision, seed=rank, t_num=args.t_num)
    job64 = make_job("fp64", seed=rank, t_num=args.t_num)
    grid = job.grid_size

    # accuracy: FP32-bulk against the FP64 plain path on the same sampled electrons
    acc = accuracy_report(eng, job, job64) if not args.no_fp64_compare else None

    def sync_all():
        torch.cuda.synchronize(dev)
        if world > 1:
            dist.barrier()

    # ---- device-resident timing (no spectrum copy) ------------------------------------
    for _ in range(args.warmup):
        eng.run(job, want_spectrum=False)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    lat, effs, launches, steps_total = [], [], 0, 0
    sync_all()
    with ClockSampler(local) as clk:
        t_wall = time.perf_counter()
        for i in range(args.steps):
            ev[i][0].record(stream)
            r, _, _ = eng.run(job, want_spectrum=False)
            ev[i][1].record(stream)
            effs.append(r.num_effective_traj)
            launches += r.num_kernel_launches
            steps_total += r.num_steps
        sync_all()
        t_wall = time.perf_counter() - t_wall
    ms = [a.elapsed_time(b) for a, b in ev]
    t_max = torch.tensor([sum(ms)], device=dev)
    if world > 1:
        dist.all_reduce(t_max, op=dist.ReduceOp.MAX)
    eff_total = torch.tensor([float(sum(effs))], device=dev)
    if world > 1:
        dist.all_reduce(eff_total)
    value = eff_total.item() / (t_max.item() / 1e3)

    # kernel-level timing of the bulk integrator for the roofline
    stages = stage_times(eng, job)
    kern_ms = stages["integrate"]

    # ---- end to end through the C ABI with host buffers --------------------------------
    spec_host = np.zeros(grid)
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        res = abi.Result()
        res.momentum_spec = abi.dptr(spec_host)
        eng._check(eng.lib.etraj_run(eng.ctx, __import__("ctypes").byref(job), __import__("ctypes").byref(res)))
        if i >= args.warmup:
            e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_value = statistics.mean(effs) / (statistics.mean(e2e_ms) / 1e3) * world

    if rank == 0:
        peaks = measured_peaks()
        clocks = clk.summary()
        sm_mhz = clocks["sm_mhz"] or peaks.get("sm_max_mhz", 2070.0)
        n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
        fp32_peak = n_sm * 128 * 2 * (peaks.get("sm_max_mhz", 2070.0) * 1e6) / 1e12
        steps_per_job = steps_total / args.steps
        flops = steps_per_job * FLOPS_PER_STEP_SAE_2D_SCTS
        achieved = flops / (kern_ms / 1e3) / 1e12 if kern_ms else None
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.mean(ms), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 stages + f64 collection/deposit",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "effective_trajectories_per_step": statistics.mean(effs),
                       "candidates_per_step": args.t_num * 1000, "l2_flush": "outputs 1e7 x 64 B > L2",
                       "parallelism": "weak: one Monte-Carlo shard per GPU (seed = rank)"},
            "precision": args.precision,
            "fp64_plain": acc and acc["fp64_plain"],
            "speedup_fp32_bulk_vs_fp64": acc and value / world / acc["fp64_plain"]["value"],
            "pmd_rel_l2_vs_fp64": acc and acc["pmd_rel_l2_vs_fp64"],
            "accuracy": acc,
            "latency_ms": {"p50": float(np.percentile(ms, 50)), "p99": float(np.percentile(ms, 99))},
            "stages_ms": stages,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * (args.t_num + 2),
                    "d2h_bytes_per_step": 8 * grid + 64},
            "gpu_launches": launches,
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": (achieved / fp32_peak) if achieved else None, "traffic": None,
                         "kernel": "k_integrate_bulk", "kernel_ms": kern_ms,
                         "flops_per_step_attempt": FLOPS_PER_STEP_SAE_2D_SCTS,
                         "step_attempts_per_job": steps_per_job,
                         "peak_source": "nominal FP32 peak: %d SMs x 128 lanes x 2 x %d MHz (no measured "
                                        "FP32 peak is provided)" % (n_sm, peaks.get("sm_max_mhz", 2070))},
            "clocks": clocks,
            "wall_s": t_wall,
        }
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(lambda n: make_job("fp64", seed=0, t_num=n))
        print(json.dumps(line))
    eng.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


def accuracy_report(eng, job, job64):
    """PMD error of the timed path against the FP64 plain path on the same electrons,
    next to the FP64 path's own sensitivity to its tolerance (rtol 1e-6 vs 1e-7), at
    the full 1000 x 1000 resolution and after rebinning to 100 x 100 and 20 x 20."""
    res64, spec64, _ = eng.run(job64, want_spectrum=True)
    res, spec, _ = eng.run(job, want_spectrum=True)
    j7 = job64.copy()
    j7.traj_rtol = 1e-7
    _, spec64b, _ = eng.run(j7, want_spectrum=True)

    def l2(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    def rebin(P, f):
        n = int(round(math.sqrt(P.size)))
        return P.reshape(n, n).reshape(n // f, f, n // f, f).sum(axis=(1, 3))

    out = {"fp64_plain": {"value": res64.num_effective_traj / (res64.elapsed_ms / 1e3), "unit": UNIT,
                          "ms_per_step": res64.elapsed_ms},
           "pmd_rel_l2_vs_fp64": l2(spec, spec64),
           "fp64_rtol1e-7_vs_rtol1e-6_pmd_rel_l2": l2(spec64b, spec64),
           "ion_prob_rel_diff": abs(res.ion_prob - res64.ion_prob) / res64.ion_prob}
    for f in (10, 50):
        out["pmd_rel_l2_vs_fp64_rebin%d" % f] = l2(rebin(spec, f), rebin(spec64, f))
        out["fp64_rtol1e-7_vs_rtol1e-6_rebin%d" % f] = l2(rebin(spec64b, f), rebin(spec64, f))
    return out


STAGES = ("sample", "compact", "field_table", "integrate", "collect", "deposit")


def stage_times(eng, job):
    """Per-stage device times of one job (mean of 3 runs) from the library's own
    events on its stream: the integrator entry is the bulk kernel's launch alone."""
    import ctypes as C

    acc = [[] for _ in STAGES]
    for _ in range(3):
        eng.run(job, want_spectrum=False)
        buf = (C.c_double * 8)()
        k = eng.lib.etraj_stage_times(eng.ctx, buf, 8)
        for i in range(min(k, len(STAGES))):
            acc[i].append(buf[i])
    return {name: (statistics.mean(v) if v else None) for name, v in zip(STAGES, acc)}


if __name__ == "__main__":
    sys.exit(main())
