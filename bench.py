"""Throughput benchmark of the ensemble-trajectory path on GB300.

Workload (the configuration the headline metric is quoted on): SAE argon
(Tong-Lin preset, Ip = 15.76 eV), Cos2 laser 800 nm, 1.2e14 W/cm^2, 2 cycles,
circular polarization; SFA-SPANE Monte-Carlo sampling of 1e7 electrons
(1e4 time samples uniform over the pulse x 1e3 transverse momenta uniform in
[-1, 1] a.u.); SCTS phase; integration to t_final = pulse end + 2 cycles with
rtol 1e-6; coherent 1000 x 1000 momentum grid spanning +-2 a.u.

A step is one whole job: sampling, integration, collection and the
deterministic deposit.  `value` is effective trajectories per second of the
timed path with all buffers resident on the device: by default the
double-float path (precision fp32_df: Tsit5 stages, field and force as
double-float pairs on the FP32 pipe, FP64 sampling, collection and deposit),
which keeps the FP64 path's step sequence and so its momentum distribution
(PMD); --precision fp32_bulk times the plain-FP32 bulk path instead, which is
~50x faster again but changes step sequences.  `e2e` is the same metric
through the C ABI's etraj_submit / etraj_wait with host output buffers (time
samples copied in and the spectrum copied back every step).  The FP64 plain
path is run on the same job for the speed ratio and the PMD error (relative L2
of |A|^2 against the FP64 result); the other FP32 path is reported beside it.

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
from etraj_gb300 import abi, shards  # noqa: E402

METRIC = "trajectories/sec on 1 GB300 (FP32-bulk vs FP64 plain, PMD L2 <=1e-3); p50/p99 job latency"
UNIT = "trajectories/s"
WORKLOAD = ("SAE Ar, Cos2 800 nm 1.2e14 W/cm^2 2 cyc CP, SPANE Monte-Carlo 1e4 t x 1e3 kd, "
            "SCTS, t_final = pulse end + 2 cycles, rtol 1e-6, coherent 1000x1000 PMD +-2 a.u.")


def make_job(precision="fp32_bulk", seed=0, t_num=10000, kt_num=1000):
    """Headline workload: 1e7 SPANE Monte-Carlo candidates, Ar, Cos2 CP, SCTS, 1000^2."""
    laser = et.Cos2Laser(peak_int=1.2e14, wave_len=800.0, cyc_num=2, ellip=1.0)
    T = laser.Period()
    half = laser.CycNum() * T / 2  # the Cos2 envelope spans [-N T/2, N T/2]
    return et.make_job(init_cond_method="SPANE", laser=laser, target=et.get_atom("Ar"), dimension=2,
                       sample_t_intv=(-half, half), sample_t_num=t_num, traj_t_final=half + 2 * T,
                       final_p_max=(2.0, 2.0), final_p_num=(1000, 1000), sample_monte_carlo=True,
                       mc_kt_num=kt_num, mc_kd_max=1.0, traj_phase_method="SCTS", seed=seed,
                       precision=precision)


def make_job_spa_bichromatic(precision="fp32_bulk", seed=0, t_num=30000, kt_num=1000):
    """Uneven-step workload: H, counter-rotating CP 800 nm (Cos4, 8 cycles) + 400 nm
    (16 cycles), 5e13 W/cm^2 each; SPA Monte-Carlo 3D (t_num x kt_num candidates,
    3e7 in full), QTMC, coherent 256^3 PMD +-2 a.u."""
    l1 = et.Cos4Laser(peak_int=5e13, wave_len=800.0, cyc_num=8, ellip=1.0)
    l2 = et.Cos4Laser(peak_int=5e13, wave_len=400.0, cyc_num=16, ellip=-1.0)
    T = l1.Period()
    return et.make_job(init_cond_method="SPA", laser=et.BichromaticLaser(l1, l2, delay=0.0),
                       target=et.get_atom("H"), dimension=3, sample_t_intv=(-4 * T, 4 * T),
                       sample_t_num=t_num, traj_t_final=6 * T, final_p_max=(2.0, 2.0, 2.0),
                       final_p_num=(256, 256, 256), sample_monte_carlo=True, mc_kt_num=kt_num,
                       mc_kd_max=1.0, mc_kz_max=1.0, traj_phase_method="QTMC", seed=seed,
                       precision=precision)


def make_job_adk_h(precision="fp32_bulk", seed=0, t_num=2000, kt_num=None):
    """Small plain workload: H, Cos4 800 nm 1e14 W/cm^2 2 cycles LP; ADK grid of t_num
    time samples x 21 x 21 (kd, kz) in [-1, 1]; CTMC; 500 x 500 PMD +-1.5 a.u."""
    laser = et.Cos4Laser(peak_int=1e14, wave_len=800.0, cyc_num=2, ellip=0.0)
    T = laser.Period()
    return et.make_job(init_cond_method="ADK", laser=laser, target=et.get_atom("H"), dimension=3,
                       sample_t_intv=(-T, T), sample_t_num=t_num, traj_t_final=3 * T,
                       final_p_max=(1.5, 1.5, 1.0), final_p_num=(500, 500, 1), ss_kd_max=1.0,
                       ss_kd_num=21, ss_kz_max=1.0, ss_kz_num=21, traj_phase_method="CTMC",
                       seed=seed, precision=precision)


WORKLOADS = {
    "ar_spane_scts_2d": (make_job, 10000, 1000, WORKLOAD),
    "h_spa_bichromatic_3d": (make_job_spa_bichromatic, 30000, 1000,
                             "H, counter-rotating CP 800+400 nm 5e13 W/cm^2 each (Cos4, 8 cycles at "
                             "800 nm), SPA Monte-Carlo 3D, QTMC, coherent 256^3 PMD +-2 a.u."),
    "h_adk_cos4_3d": (make_job_adk_h, 2000, 441,
                      "H, Cos4 800 nm 1e14 W/cm^2 2 cycles LP, ADK grid t x 21 x 21, CTMC, "
                      "incoherent 500 x 500 PMD +-1.5 a.u."),
}


# FP32 operations of one Tsit5 step of the bulk integrator for 2D SAE SCTS, counted
# from integrate_fp32.cu (an FMA counts 2, every other arithmetic instruction 1,
# MUFU ops 1): right-hand side 52 (field 12, radius and rsqrt 14, three exponentials
# 6, bracket and force 12, phase 8) x 6 stages = 312; stage combinations
# 2*(1+2+3+4+5+6)*5 = 210; error estimate 5*(2*7+6) = 100; compensated update
# 5*8 = 40; clock, controller and bookkeeping ~40.  Total 702 per step attempt.
FLOPS_PER_STEP_SAE_2D_SCTS = 702
# DRAM bytes (read + write) of the bulk integrator's round-0 launch per electron on
# this workload, from one ncu capture of a 2e6-candidate case (24.91 MB for 8.17e5
# electrons); traffic grows with the electrons.
INTEGRATOR_DRAM_BYTES_PER_ELECTRON = 30.48
# The double-float integrator (start-up and main pass) on the same workload, from one
# ncu capture of both passes on a 4e5-candidate case (400 time samples: 161,722
# electrons, 6,489,343 step attempts): FP32 thread instructions
# (smsp__sass_thread_inst_executed_op_fp32_pred_on: 4.07e9 start-up + 3.928e10
# main; 68 % FADD, 21 % FFMA, 8 % FMUL) per step attempt, and DRAM bytes (read +
# write, 14.53 MB + 16.04 MB) per electron.  At that size the carry buffer between
# the passes (116 B per electron) stays in L2; at full size it adds about that much
# per electron again.  FMA-pipe issue (sm__inst_executed_pipe_fma, warp
# instructions against 4 per SM and cycle) was 35.3 % (start-up) and 41.5 % (main).
DF_FP32_INST_PER_STEP = 6717
DF_DRAM_BYTES_PER_ELECTRON = 189.0
DF_FMA_PIPE_ISSUE_NCU = {"start_up": 0.348, "main": 0.505}


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


def cpu_baseline(job_fn, t_full=10000, seconds_target=15.0):
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
        if dt > seconds_target / 4 or t_num >= t_full:
            break
        t_num = min(t_full, int(t_num * max(2.0, seconds_target / 3 / max(dt, 1e-3))))
    return {"value": sc["num_effective"] / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d of %d time samples (%d effective trajectories, %.1f s)"
                      % (t_num, t_full, int(sc["num_effective"]), dt)}


def run_reference(args):
    rank, world, _ = rank_env()
    if rank != 0:
        return 0
    maker, t_full, _, workload_text = WORKLOADS[args.workload]
    job_fn = lambda n: maker("fp64", seed=0, t_num=n)  # noqa: E731
    # each step a bounded sample: about 120 s for the whole run, at most ~3 s a step
    per_step = min(3.0, 120.0 / max(1, args.steps + args.warmup))
    base = cpu_baseline(job_fn, t_full, seconds_target=4.0 * per_step)
    n = int(base["sample"].split(" ")[0])
    times, effs = [], []
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle

    sys.path.pop(0)
    for i in range(args.warmup + args.steps):
        job = maker("fp64", seed=i, t_num=n)
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
            "data": "synthetic", "config": {"workload": workload_text, "sample": base["sample"]},
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
    ap.add_argument("--workload", default="ar_spane_scts_2d", choices=sorted(WORKLOADS),
                    help="ar_spane_scts_2d is the headline workload; the others are the uneven-step "
                         "SPA workload and the small ADK workload")
    ap.add_argument("--t-num", type=int, default=None,
                    help="time samples (default: the workload's full size)")
    ap.add_argument("--precision", default="fp32_df", choices=["fp32_df", "fp32_bulk", "fp64"],
                    help="path timed as `value` (fp32_df: the double-float path that keeps the FP64 "
                         "step sequence; fp32_bulk: plain FP32; fp64 profiles the plain kernel)")
    ap.add_argument("--no-multi-instance", action="store_true",
                    help="skip the 64-instance batched intensity scan")
    ap.add_argument("--no-serving", action="store_true",
                    help="skip the serving-loop replay (512 Poisson arrivals at 20/s)")
    ap.add_argument("--no-scheduling", action="store_true",
                    help="skip the static-assignment vs work-stealing comparison of the bulk integrator")
    ap.add_argument("--no-fp64-compare", action="store_true",
                    help="skip the FP64 run used for the speed ratio and PMD error (profiling)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import torch.distributed as dist

    rank, world, local = rank_env()
    torch.cuda.set_device(local)  # before the process group, so NCCL binds this rank's GPU
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = torch.device("cuda", local)
    eng = et.Engine(device=local)
    stream = torch.cuda.Stream(device=dev)
    eng.set_stream(stream.cuda_stream)

    maker, t_full, kt_per_t, workload_text = WORKLOADS[args.workload]
    if args.t_num is None:
        args.t_num = t_full
    headline = (args.workload == "ar_spane_scts_2d")
    # one Monte-Carlo shard per rank (seed = rank), weight 1/world in a merge
    job, shard_w = shards.shard_job(maker(args.precision, seed=0, t_num=args.t_num), rank, world)
    job64, _ = shards.shard_job(maker("fp64", seed=0, t_num=args.t_num), rank, world)
    other = {"fp32_df": "fp32_bulk", "fp32_bulk": "fp32_df"}.get(args.precision)
    job_other = shards.shard_job(maker(other, seed=0, t_num=args.t_num), rank, world)[0] if other else None
    grid = job.grid_size

    # accuracy: the timed path (and the other FP32 path) against the FP64 plain path
    # on the same sampled electrons
    acc = accuracy_report(eng, job, job64, job_other) if not args.no_fp64_compare else None
    tstats = trajectory_stats(eng, job, job64) if not args.no_fp64_compare else None

    def sync_all():
        torch.cuda.synchronize(dev)
        if world > 1:
            dist.barrier()

    # ---- device-resident timing (no spectrum copy) ------------------------------------
    # Jobs go through the asynchronous entry points with up to 4 in flight, so the
    # host set-up of one job overlaps the kernels of the one before; events on the
    # library's stream bracket the timed sequence, and each job's own device time
    # (its start/done events inside the library) gives the latency percentiles.
    for _ in range(args.warmup):
        eng.run(job, want_spectrum=False)
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    lat, effs, launches, steps_total = [], [], 0, 0
    sync_all()
    with ClockSampler(local) as clk:
        t_wall = time.perf_counter()
        t_start.record(stream)
        inflight = []
        for i in range(args.steps):
            res = abi.Result()
            inflight.append((eng.submit(job, res), res))
            if len(inflight) == 4 or i == args.steps - 1:
                if i == args.steps - 1:
                    t_end.record(stream)
                while inflight and (len(inflight) == 4 or i == args.steps - 1):
                    tk, r = inflight.pop(0)
                    eng.wait(tk, r)
                    lat.append(r.elapsed_ms)
                    effs.append(r.num_effective_traj)
                    launches += r.num_kernel_launches
                    steps_total += r.num_steps
        sync_all()
        t_wall = time.perf_counter() - t_wall
    ms = lat
    t_local = t_start.elapsed_time(t_end) / 1e3
    if world > 1:
        _, t_slowest, value = shards.aggregate_throughput(sum(effs), t_local)
    else:
        t_slowest, value = t_local, sum(effs) / t_local

    # kernel-level timing of the integrator for the roofline
    stages = stage_times(eng, job)
    kern_ms = stages["integrate"]

    # ---- end to end through the C ABI with host buffers --------------------------------
    # The same jobs through etraj_submit / etraj_wait, up to 4 in flight, each with
    # its own host spectrum buffer: the library copies the time samples from the
    # host, stages each spectrum in pinned memory and copies it into the caller's
    # buffer when the job is waited on, so every host<->device copy and that host
    # copy are inside the timed region.
    spec_host = [np.zeros(grid) for _ in range(4)]

    def e2e_pass(steps):
        inflight, effs_done = [], []
        for i in range(steps):
            res = abi.Result()
            res.momentum_spec = abi.dptr(spec_host[i % 4])
            inflight.append((eng.submit(job, res), res))
            while inflight and (len(inflight) == 4 or i == steps - 1):
                tk, r = inflight.pop(0)
                eng.wait(tk, r)
                effs_done.append(r.num_effective_traj)
        return effs_done

    e2e_pass(max(args.warmup, 4))  # the same pattern untimed: the pinned staging blocks exist
    sync_all()
    t_e2e = time.perf_counter()
    e2e_effs = e2e_pass(args.steps)
    t_e2e = time.perf_counter() - t_e2e
    if world > 1:
        _, _, e2e_value = shards.aggregate_throughput(sum(e2e_effs), t_e2e)
    else:
        e2e_value = sum(e2e_effs) / t_e2e

    # N > 1 (untimed): the shards merged into one job's result by one all-reduce
    merged = None
    if world > 1:
        coh = shards.is_coherent(job)
        r1, s1, a1 = eng.run(job, want_spectrum=not coh, want_amplitude=coh)
        mspec, mion, munc, meff = shards.merge_shards(r1, s1, a1, shard_w, coh)
        merged = {"num_effective_traj": meff, "ion_prob": mion, "ion_prob_uncollected": munc,
                  "momentum_spec_sum": float(mspec.sum())}

    if rank == 0:
        peaks = measured_peaks()
        clocks = clk.summary()
        sm_mhz = clocks["sm_mhz"] or peaks.get("sm_max_mhz", 2070.0)
        n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
        sm_max = peaks.get("sm_max_mhz", 2070.0)
        steps_per_job = steps_total / args.steps
        eff_mean = statistics.mean(effs)
        if args.precision == "fp32_df":
            # FP32-pipe issue: thread instructions per second against 128 lanes x SMs x clock
            per_step = DF_FP32_INST_PER_STEP
            achieved = (steps_per_job * per_step / (kern_ms / 1e3) / 1e12
                        if (kern_ms and headline and per_step) else None)
            roof = {"bound": "fp32_issue", "achieved": achieved, "peak": n_sm * 128 * sm_max * 1e6 / 1e12,
                    "unit": "T FP32-pipe thread instructions/s",
                    "traffic": (DF_DRAM_BYTES_PER_ELECTRON * eff_mean)
                    if (headline and DF_DRAM_BYTES_PER_ELECTRON) else None,
                    "kernel": "k_integrate_df (start-up + main pass)", "kernel_ms": kern_ms,
                    "fp32_inst_per_step_attempt": per_step, "step_attempts_per_job": steps_per_job,
                    "fma_pipe_issue_frac_ncu": DF_FMA_PIPE_ISSUE_NCU,
                    "peak_source": "nominal FP32 issue: %d SMs x 128 lanes x %d MHz (no measured FP32 "
                                   "peak is provided)" % (n_sm, sm_max)}
        else:
            flops = steps_per_job * FLOPS_PER_STEP_SAE_2D_SCTS
            # the flop count per step is the headline workload's (2D SAE SCTS)
            achieved = flops / (kern_ms / 1e3) / 1e12 if (kern_ms and headline) else None
            roof = {"bound": "fp32", "achieved": achieved, "peak": n_sm * 128 * 2 * sm_max * 1e6 / 1e12,
                    "unit": "TFLOP/s",
                    "traffic": (INTEGRATOR_DRAM_BYTES_PER_ELECTRON * eff_mean) if headline else None,
                    "kernel": "k_integrate_bulk" if args.precision == "fp32_bulk" else "k_integrate_fp64",
                    "kernel_ms": kern_ms, "flops_per_step_attempt": FLOPS_PER_STEP_SAE_2D_SCTS,
                    "step_attempts_per_job": steps_per_job,
                    "peak_source": "nominal FP32 peak: %d SMs x 128 lanes x 2 x %d MHz (no measured "
                                   "FP32 peak is provided)" % (n_sm, sm_max)}
        roof["frac"] = (roof["achieved"] / roof["peak"]) if roof["achieved"] else None
        dtype = {"fp32_df": "f32 pairs (double-float) stages + f64 sampling/collection/deposit",
                 "fp32_bulk": "f32 stages + f64 phase/deposit", "fp64": "f64"}[args.precision]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_slowest / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic",
            "config": {"workload": workload_text, "effective_trajectories_per_step": statistics.mean(effs),
                       "candidates_per_step": args.t_num * kt_per_t,
                       "l2_flush": "per-electron buffers of every step exceed L2 (1e7 x ~100 B)",
                       "parallelism": "weak: one Monte-Carlo shard per GPU (seed = rank)"},
            "precision": args.precision,
            "fp64_plain": acc and acc["fp64_plain"],
            "speedup_vs_fp64": acc and value / world / acc["fp64_plain"]["value"],
            "pmd_rel_l2_vs_fp64": acc and acc["pmd_rel_l2_vs_fp64"],
            "pmd_gate_1e-3_met": acc and acc["pmd_rel_l2_vs_fp64"] <= 1e-3,
            "accuracy": acc,
            "trajectory_stats": tstats,
            "merged_shards": merged,
            "latency_ms": {"p50": float(np.percentile(ms, 50)), "p99": float(np.percentile(ms, 99))},
            "stages_ms": stages,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * (args.t_num + 2),
                    "d2h_bytes_per_step": 8 * grid + 64},
            "gpu_launches": launches,
            "roofline": roof,
            "clocks": clocks,
            "wall_s": t_wall,
        }
        if not args.no_multi_instance and world == 1:
            line["multi_instance"] = multi_instance_report(eng)
            # the autotuner shapes the bulk integrator: tuned against fixed on the bulk job
            job_bulk = job if args.precision == "fp32_bulk" else maker("fp32_bulk", seed=0, t_num=args.t_num)
            line["autotune"] = autotune_report(eng, job_bulk, multi_instance_jobs()[0])
            line["graphs"] = graphs_report(lambda n: maker(args.precision, seed=rank, t_num=n or args.t_num))
        if not args.no_scheduling and world == 1:
            job_bulk = job if args.precision == "fp32_bulk" else maker("fp32_bulk", seed=0, t_num=args.t_num)
            line["scheduling"] = scheduling_report(job_bulk)
        if not args.no_serving and world == 1:
            line["serving"] = serving_report()
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(lambda n: maker("fp64", seed=0, t_num=n), t_full)
        print(json.dumps(line))
    eng.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


def accuracy_report(eng, job, job64, job_other=None):
    """PMD error of the timed path against the FP64 plain path on the same electrons,
    next to the FP64 path's own sensitivity to its tolerance (rtol 1e-6 vs 1e-7), at
    the full 1000 x 1000 resolution and after rebinning to 100 x 100 and 20 x 20;
    job_other (the other FP32 path) gets its speed (5 runs) and PMD error beside it."""
    res64, spec64, _ = eng.run(job64, want_spectrum=True)
    res, spec, _ = eng.run(job, want_spectrum=True)
    j7 = job64.copy()
    j7.traj_rtol = 1e-7
    _, spec64b, _ = eng.run(j7, want_spectrum=True)

    def l2(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    dims = [int(job.final_p_num[d]) for d in range(job.dimension)]

    def rebin(P, f):
        # Julia column-major grid: x fastest
        a = P.reshape(tuple(reversed(dims)))
        for ax in range(a.ndim):
            if a.shape[ax] > 1:
                a = np.add.reduceat(a, np.arange(0, a.shape[ax], f), axis=ax)
        return a.ravel()

    out = {"fp64_plain": {"value": res64.num_effective_traj / (res64.elapsed_ms / 1e3), "unit": UNIT,
                          "ms_per_step": res64.elapsed_ms},
           "pmd_rel_l2_vs_fp64": l2(spec, spec64),
           "fp64_rtol1e-7_vs_rtol1e-6_pmd_rel_l2": l2(spec64b, spec64),
           "ion_prob_rel_diff": abs(res.ion_prob - res64.ion_prob) / res64.ion_prob}
    for f in (10, 50):
        out["pmd_rel_l2_vs_fp64_rebin%d" % f] = l2(rebin(spec, f), rebin(spec64, f))
        out["fp64_rtol1e-7_vs_rtol1e-6_rebin%d" % f] = l2(rebin(spec64b, f), rebin(spec64, f))
    if job_other is not None:
        eng.run(job_other, want_spectrum=False)
        ms = []
        for _ in range(5):
            r, _, _ = eng.run(job_other, want_spectrum=False)
            ms.append(r.elapsed_ms)
        r, so, _ = eng.run(job_other, want_spectrum=True)
        name = {abi.PRECISION_FP32_BULK: "fp32_bulk", abi.PRECISION_FP32_DF: "fp32_df"}[job_other.precision]
        out[name] = {
            "value": r.num_effective_traj / (min(ms) / 1e3), "unit": UNIT, "ms_per_step": min(ms),
            "pmd_rel_l2_vs_fp64": l2(so, spec64), "pmd_rel_l2_vs_fp64_rebin50": l2(rebin(so, 50), rebin(spec64, 50)),
            "speedup_vs_fp64": res64.elapsed_ms / min(ms)}
    return out


def trajectory_stats(eng, job, job64):
    """The workload's per-trajectory character: the share of survivors that return
    within r < 5 a.u. of the core (least |r| over the FP64 path's accepted steps)
    and the distribution of Tsit5 step attempts per survivor on both paths, with
    power-of-two bins (bin k counts 2^k <= steps < 2^(k+1))."""
    eng.keep_final_states(True)
    try:
        r64, _, _ = eng.run(job64)
        rmin = eng.dump_min_radius(r64.num_effective_traj)
        s64 = eng.dump_step_counts(r64.num_effective_traj)
        r32, _, _ = eng.run(job)
        s32 = eng.dump_step_counts(r32.num_effective_traj)
    finally:
        eng.keep_final_states(False)

    def hist(s):
        if s.size == 0:
            return None
        bins = np.bincount(np.floor(np.log2(np.maximum(s, 1))).astype(np.int64))
        return {"mean": float(s.mean()), "p50": float(np.percentile(s, 50)), "p99": float(np.percentile(s, 99)),
                "max": int(s.max()), "log2_bins": [int(x) for x in bins]}

    return {"frac_rmin_below_5": float(np.mean(rmin < 5.0)) if rmin.size else None,
            "steps_fp64": hist(s64), "steps_timed_path": hist(s32),
            "step_counts_differing_from_fp64": int(np.sum(s32 != s64)) if s32.shape == s64.shape else None}


def serving_requests(n=512, rate=20.0, seed=2024, precision="fp32_bulk"):
    """The serving workload: n requests with Poisson arrivals at `rate` per second,
    each a random mix of target {H, Ar}, laser {Cos4 LP, Cos2 CP, counter-rotating
    CP bichromatic (lambda, lambda/2)}, wavelength U(400, 1600) nm, intensity
    log-U(5e13, 3e14) W/cm^2, 1-8 cycles, sampler {ADK, SPANE}, phase {CTMC, QTMC,
    SCTS}, log-U(1e4, 3e7) Monte-Carlo candidates and a 2D grid of 256^2-1000^2."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
    reqs = []
    for i in range(n):
        lam = rng.uniform(400.0, 1600.0)
        inten = float(np.exp(rng.uniform(np.log(5e13), np.log(3e14))))
        cyc = int(rng.integers(1, 9))
        kind = int(rng.integers(0, 3))
        if kind == 0:
            laser = et.Cos4Laser(peak_int=inten, wave_len=lam, cyc_num=cyc, ellip=0.0)
        elif kind == 1:
            laser = et.Cos2Laser(peak_int=inten, wave_len=lam, cyc_num=cyc, ellip=1.0)
        else:
            laser = et.BichromaticLaser(et.Cos4Laser(peak_int=inten, wave_len=lam, cyc_num=cyc, ellip=1.0),
                                        et.Cos4Laser(peak_int=inten, wave_len=lam / 2, cyc_num=2 * cyc,
                                                     ellip=-1.0), delay=0.0)
        T = 2 * np.pi * lam / 45.563352525
        half = cyc * T / 2 if kind == 1 else cyc * T
        ncand = float(np.exp(rng.uniform(np.log(1e4), np.log(3e7))))
        t_num = max(10, int(round(ncand / 1000)))
        grid = int(rng.integers(256, 1001))
        job = et.make_job(init_cond_method=("ADK", "SPANE")[int(rng.integers(0, 2))], laser=laser,
                          target=et.get_atom(("H", "Ar")[int(rng.integers(0, 2))]), dimension=2,
                          sample_t_intv=(-half, half), sample_t_num=t_num, traj_t_final=half + 2 * T,
                          final_p_max=(2.0, 2.0), final_p_num=(grid, grid), sample_monte_carlo=True,
                          mc_kt_num=1000, mc_kd_max=1.0,
                          traj_phase_method=("CTMC", "QTMC", "SCTS")[int(rng.integers(0, 3))],
                          seed=i, precision=precision)
        reqs.append(job)
    return arrivals, reqs


def serving_report(n=512, rate=20.0, slots=8, fp64_seconds=20.0, precision="fp32_bulk"):
    """Replays the request stream in real time against an etraj server (at
    `precision`) and reports arrival-to-result latency and aggregate throughput;
    then, unless fp64_seconds is 0, serves the stream's first requests one at a
    time on the FP64 path, for about `fp64_seconds` (a request's time is set by
    its slowest trajectory)."""
    arrivals, reqs = serving_requests(n, rate, precision=precision)
    srv = et.Server(device=0, slots=slots)
    # warm-up: one small job per slot
    for t in [srv.submit(reqs[k]) for k in range(slots)]:
        srv.wait(t, timeout=600.0)
    lat, effs, pending = [], [], {}
    t0 = time.perf_counter()
    i = 0
    max_running = max_queued = 0
    while i < n or pending:
        now = time.perf_counter() - t0
        while i < n and arrivals[i] <= now:
            pending[srv.submit(reqs[i])] = arrivals[i]
            i += 1
        running, queued, _ = srv.stats()
        max_running, max_queued = max(max_running, running), max(max_queued, queued)
        done = []
        for tk, arr in pending.items():
            out = srv.poll(tk)
            if out is not None:
                lat.append(time.perf_counter() - t0 - arr)
                effs.append(out[0].num_effective_traj)
                done.append(tk)
        for tk in done:
            del pending[tk]
        if not done:
            time.sleep(0.0005)
    span = time.perf_counter() - t0 - arrivals[0]
    srv.close()
    lat_ms = 1e3 * np.array(lat)
    out = {"precision": precision, "requests": n, "arrival_rate_per_s": rate, "slots": slots,
           "latency_ms": {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99)),
                          "max": float(lat_ms.max())},
           "trajectories_per_s": float(sum(effs) / span), "effective_trajectories": int(sum(effs)),
           "span_s": float(span), "max_running": max_running, "max_queued": max_queued,
           "workload": serving_requests.__doc__.split("\n\n")[0].replace("\n    ", " ")}
    if fp64_seconds > 0:
        eng = et.Engine(device=0)
        fp64_ms, fp64_eff = [], []
        for job in reqs:
            j = job.copy()
            j.precision = abi.PRECISION_FP64
            t1 = time.perf_counter()
            r, _, _ = eng.run(j, want_spectrum=True)
            fp64_ms.append(1e3 * (time.perf_counter() - t1))
            fp64_eff.append(r.num_effective_traj)
            if sum(fp64_ms) > 1e3 * fp64_seconds:
                break
        eng.close()
        out["fp64_one_at_a_time"] = {"requests": len(fp64_ms),
                                     "trajectories_per_s": sum(fp64_eff) / (sum(fp64_ms) / 1e3),
                                     "mean_service_ms": float(np.mean(fp64_ms)),
                                     "offered_load_vs_capacity": float(rate * np.mean(fp64_ms) / 1e3)}
    return out


def multi_instance_jobs(n=64, seed=7):
    """Focal-volume intensity scan: n instances of Ar, Gaussian 800 nm (8 cycles
    FWHM) linear polarization, peak intensity log-U(5e13, 4e14) W/cm^2,
    log-U(1e4, 2e6) ADK Monte-Carlo candidates in 3D (kd, kz), SCTS, each with
    a 500 x 500 x 1 grid +-2 a.u.; weights I^-1.5 (a focal volume's dV/dI shape)."""
    rng = np.random.default_rng(seed)
    jobs, ints = [], []
    for i in range(n):
        inten = float(np.exp(rng.uniform(np.log(5e13), np.log(4e14))))
        count = float(np.exp(rng.uniform(np.log(1e4), np.log(2e6))))
        T = 2 * np.pi * 800.0 / 45.563352525
        laser = et.GaussianLaser(peak_int=inten, wave_len=800.0, FWHM_duration=8 * T, ellip=0.0)
        fw = 8 * T
        jobs.append(et.make_job(init_cond_method="ADK", laser=laser, target=et.get_atom("Ar"), dimension=3,
                                sample_t_intv=(-1.5 * fw, 1.5 * fw), sample_t_num=max(10, int(round(count / 1000))),
                                traj_t_final=1.5 * fw + 2 * T, final_p_max=(2.0, 2.0, 1.0),
                                final_p_num=(500, 500, 1), sample_monte_carlo=True, mc_kt_num=1000,
                                mc_kd_max=1.0, mc_kz_max=1.0, traj_phase_method="SCTS", seed=1000 + i,
                                precision="fp32_bulk"))
        ints.append(inten)
    ints = np.array(ints)
    return jobs, (ints / ints.max()) ** -1.5


def multi_instance_report(eng):
    """The 64-instance scan as one batch (one integrator launch whose work stealing
    spans every instance, plus the weighted PMD) against the same 64 jobs run one
    after another; device times from the library's events.  The first call of a
    batch grows the buffers and tunes the batch's launch shape (`cold`); the
    second runs directly and the third replays the CUDA graph captured on the
    second, which is the timed call."""
    jobs, w = multi_instance_jobs()
    walls = []
    for _ in range(3):
        t0 = time.perf_counter()
        outs, wsum = eng.run_batch(jobs, want_spectrum=True, weights=w)
        walls.append(time.perf_counter() - t0)
    wall_batch = walls[-1]
    eff = sum(r.num_effective_traj for r, _, _ in outs)
    dev_batch = outs[0][0].elapsed_ms
    t0 = time.perf_counter()
    dev_seq = 0.0
    for job in jobs:
        r, _, _ = eng.run(job, want_spectrum=True)
        dev_seq += r.elapsed_ms
    wall_seq = time.perf_counter() - t0
    return {"instances": len(jobs), "effective_trajectories": int(eff),
            "batched": {"device_ms": dev_batch, "wall_ms": 1e3 * wall_batch,
                        "wall_ms_cold_direct_graph": [1e3 * x for x in walls],
                        "trajectories_per_s": eff / (dev_batch / 1e3), "kernel_launches": outs[0][0].num_kernel_launches,
                        "graph_launches_per_batch": 1},
            "one_job_at_a_time": {"device_ms": dev_seq, "wall_ms": 1e3 * wall_seq,
                                  "trajectories_per_s": eff / (dev_seq / 1e3)},
            "weighted_pmd_sum": float(wsum.sum()),
            "workload": multi_instance_jobs.__doc__.replace("\n    ", " ")}


def autotune_report(eng, job, batch_jobs):
    """Integrator time with the autotuner's launch shape against the fixed 256 x 2 x 4,
    for the headline job and for the 64-instance batch."""
    fixed = et.Engine(device=0)
    fixed.set_autotune(False)
    out = {}
    for name, run in (("headline", lambda e: e.run(job, want_spectrum=False)),
                      ("multi_instance", lambda e: e.run_batch(batch_jobs, want_spectrum=False))):
        row = {}
        for tag, e in (("tuned", eng), ("fixed", fixed)):
            run(e)
            vals = []
            for _ in range(3):
                run(e)
                import ctypes as C
                buf = (C.c_double * 8)()
                if e.lib.etraj_stage_times(e.ctx, buf, 8) > 3:
                    vals.append(buf[3])
            row[tag + "_integrate_ms"] = statistics.mean(vals) if vals else None
        j0 = job if name == "headline" else batch_jobs[0]
        t, b, r, tuned = eng.bulk_tile(j0.dimension, j0.traj_phase_method, j0.target.kind, name != "headline")
        chunk, _ = eng.bulk_step_chunk(j0.dimension, j0.traj_phase_method, j0.target.kind, name != "headline")
        row["tile"] = {"threads": t, "blocks_per_sm": b, "refill_min": r, "step_chunk": chunk, "tuned": tuned}
        out[name] = row
    fixed.close()
    return out


def scheduling_report(job):
    """The bulk integrator with work stealing (persistent grid, warp-aggregated
    refills, rounds) against static assignment (one electron per lane, as the
    plain kernel schedules), same precision and same bits; integrator device time
    (mean of 3 runs) and the spread of step attempts per electron that work
    stealing absorbs."""
    import ctypes as C
    out = {}
    steps = None
    for tag, static in (("work_stealing", False), ("static_assignment", True)):
        e = et.Engine(device=0)
        e.set_static_assignment(static)
        e.keep_final_states(True)
        e.run(job, want_spectrum=False)
        vals = []
        for _ in range(3):
            r, _, _ = e.run(job, want_spectrum=False)
            buf = (C.c_double * 8)()
            if e.lib.etraj_stage_times(e.ctx, buf, 8) > 3:
                vals.append(buf[3])
        if steps is None:
            steps = e.dump_step_counts(r.num_effective_traj)
        e.close()
        ms = statistics.mean(vals)
        out[tag] = {"integrate_ms": ms, "trajectories_per_s": r.num_effective_traj / (ms / 1e3)}
    out["speedup"] = out["static_assignment"]["integrate_ms"] / out["work_stealing"]["integrate_ms"]
    if steps is not None and steps.size:
        out["steps_per_electron"] = {"mean": float(steps.mean()), "p50": float(np.percentile(steps, 50)),
                                     "p99": float(np.percentile(steps, 99)), "max": int(steps.max()),
                                     "min": int(steps.min())}
    return out


def graphs_report(job_fn):
    """Per-job device and wall time with and without CUDA-graph replay, for the
    headline job and a 1e5-candidate job of the same workload (where launch
    overhead matters)."""
    out = {}
    for name, t_num in (("1e5_candidates", 100), ("headline", None)):
        job = job_fn(t_num)
        row = {}
        for tag, on in (("direct", False), ("graph", True)):
            e = et.Engine(device=0)
            e.set_graphs(on)
            for _ in range(3):
                e.run(job, want_spectrum=False)
            dev, wall = [], []
            for _ in range(20):
                t0 = time.perf_counter()
                r, _, _ = e.run(job, want_spectrum=False)
                wall.append(1e3 * (time.perf_counter() - t0))
                dev.append(r.elapsed_ms)
            e.close()
            row[tag] = {"device_ms": statistics.median(dev), "wall_ms": statistics.median(wall)}
        out[name] = row
    return out


STAGES = ("sample", "compact", "field_table", "integrate", "collect", "deposit")


def stage_times(eng, job):
    """Per-stage device times of one job (mean of 3 runs) from the library's own
    events on its stream: the integrator entry is its kernels' launches alone."""
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
