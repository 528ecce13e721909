"""Benchmark: Schwarzschild shadow sweep + concurrent bisections (ray-steps/s),
with the other workloads of the task measured beside it.

Headline workload (one step), Schwarzschild M = 1 (horizon_pad 1.001,
escape_radius 1000), observer r_obs = 20M, RK4 step 0.01, cap 200,000 steps
(bin/validate_shadow.rs settings):
  * sweep: 2^20 equatorial rays with launch angle alpha ~ U[10 deg, 20 deg]
    (seeded), each classified captured / escaped;
  * 64 concurrent 40-iteration bisections of alpha_c from seeded brackets
    lo ~ U[13, 14] deg, hi ~ U[14.5, 15.5] deg.
At r_obs = 20M the critical angle is 14.269 deg, inside both ranges (at 30M it
is 9.63 deg, outside them; the 30M variant with its own ranges is a leg below).
Inputs are synthetic and seeded.

value = useful ray-steps (sweep steps + the bisections' sequential-path steps)
per second of device time with inputs resident in HBM (mixed FP32/FP64 path).
The mixed path runs the bisection rounds first and then the sweep on the whole
GPU (the rounds take a few ms alone); the FP64 path runs them beside the
sweep (`--schedule`).
Beside it, in the same JSON line (rank 0, full workload):
  accuracy      mixed vs FP64 classes on 1/32 of the sweep, traced with the
                timed planar step, disagreements settled by the FP64 arbiter
                (geon_gb300.accuracy); escape directions, null drift, b_c;
  fp64_path     the plain FP64 path (the reference's arithmetic) on every 32nd
                sweep ray + the 64 bisections, 5 device-timed steps: ray-steps/s
                and p50/p99 step latency; fp64fast_path: GEON_FP64_FAST, 1 step;
  e2e           the host API with pinned buffers, copies inside, repeated;
  cpu_baseline  the C++ restatement of the reference on the host cores;
  config1       256^2 Schwarzschild render (r 30M, fov 60, h 0.05, cap 20000):
                FP64, FP64_FAST, mixed; the reference's own CUDA kernel at its
                escape radius (1000M) beside FP64 and FP64_FAST there;
  config3       2048^2 Alcubierre and Morris-Thorne renders (mixed, full
                images) and their FP64 classes on a row sample;
  config4       128^3 Alcubierre curvature grid (Einstein + 16 T(k, k)), FP64;
  config2_r30   the sweep + bisections at r_obs = 30M (alpha ~ U[5, 15] deg,
                brackets around 9.63 deg).
`--workload serve|render|exotic|curvature` prints one of those as its own line
(serve: the Poisson request stream through geon_gb300.Server).
`--impl reference` times the CPU restatement of the reference (oracle/) on
the host cores instead.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time
import traceback

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

R_OBS = 20.0
STEP = 0.01
MAX_STEPS = 200000
N_SWEEP = 1 << 20
N_BRACKETS = 64
ITERS = 40
SCHW = [1.0, 1.001, 1000.0]
# Overlap schedule only: slots of 128 threads per SM the persistent sweep grid
# leaves to the concurrent bisection rounds. The bisection is a chain of
# dependent rounds (latency-bound), the sweep throughput-bound. With the early
# class decision a round ends once its slowest near-critical ray settles, so 2
# of the 8 slots per SM keep the bisections well inside the sweep (measured on
# GB300, sweep / bisection ms: 320 / 314 at 0, 327 / 212 at 1, 326 / 97 at 2,
# 337 / 27 at 4, 448 / 13 at 6). The serial schedule (the mixed path's
# default) beats all of these: the rounds alone take 6 ms.
RESERVE = 2
BISECT_RAYS = 16384  # speculative width of a bisection round (geon_set_bisect_rays_per_round)
ALG_FLOPS_PER_STEP = 268  # 4 closed-form Schwarzschild RHS (41 flops each) + 104 RK4 combine flops
# The mixed path's closed-form right-hand sides (metric_analytic.cuh) for the
# config-3 metrics, counted by hand (a fused multiply-add counts 2): Alcubierre
# rhs_stage 60 flops besides one division, one square root and two tanh;
# Morris-Thorne rhs_planar (the orbit-plane step) 7 besides one division; plus
# the 104 combine flops of the reference's RK4 step.
MIXED_CLOSED_FORM_FLOPS_PER_STEP = {"alcubierre": 4 * 60 + 104, "morris_thorne": 4 * 7 + 104}
CURV_FLOPS_PER_POINT = 20000  # Alcubierre: 9 FD Christoffel evaluations, Riemann, contractions, 16 T(k, k)
B_C = 3.0 * np.sqrt(3.0)
# 30M variant: alpha_c = asin(3 sqrt(3) sqrt(1 - 2/30) / 30) = 9.633 deg
R_OBS_30 = 30.0


def workload(seed):
    rng = np.random.default_rng(seed)
    alpha = np.radians(rng.uniform(10.0, 20.0, N_SWEEP))
    lo = np.radians(rng.uniform(13.0, 14.0, N_BRACKETS))
    hi = np.radians(rng.uniform(14.5, 15.5, N_BRACKETS))
    return alpha, lo, hi


def workload_r30(seed):
    rng = np.random.default_rng(seed)
    alpha = np.radians(rng.uniform(5.0, 15.0, N_SWEEP))
    lo = np.radians(rng.uniform(9.0, 9.5, N_BRACKETS))
    hi = np.radians(rng.uniform(9.8, 10.3, N_BRACKETS))
    return alpha, lo, hi


def shard_totals(dist, t_local, units_local, device="cpu"):
    """The job's (time, units) over ranks: the slowest rank's time, the sum of
    their units (geon_gb300.shard.job_totals)."""
    from geon_gb300 import shard
    return shard.job_totals(dist, t_local, units_local, device)


def rank_workload(rank, seed=0x5EED):
    """The headline workload of one rank: its own seeded sweep and brackets."""
    from geon_gb300 import shard
    return workload(shard.rank_seed(seed, rank))


def b_of(alpha, r_obs=R_OBS):
    return r_obs * np.sin(alpha) / np.sqrt(1.0 - 2.0 / r_obs)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
                power.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [s for s in sm if s > 0.5 * max(sm)]
        return {"sm_mhz": float(np.median(load)), "sm_max_mhz": max(smax), "samples": len(sm),
                "power_w_max": max(power), "reasons": sorted(reasons)}


def cpu_sample_rate(orc, alpha, n, threads, r_obs=R_OBS):
    """Oracle (CPU restatement of the reference) on a uniform sample of the sweep."""
    sample = alpha[:: max(1, len(alpha) // n)][:n]
    t0 = time.perf_counter()
    term, steps = orc.shadow_classify(SCHW, r_obs, sample, STEP, MAX_STEPS, math=orc.LIBM, nthreads=threads)
    dt = time.perf_counter() - t0
    return float(steps.sum()) / dt, dt, int(steps.sum()), len(sample)


def run_reference(args, rank, world):
    if rank != 0:
        return
    from oracle import oracle as orc
    alpha, lo, hi = workload(0x5EED)
    threads = orc.hardware_threads()
    n = args.cpu_rays
    rates = []
    for i in range(args.warmup + args.steps):
        rate, dt, st, ns = cpu_sample_rate(orc, np.roll(alpha, 7919 * i), n, threads)
        if i >= args.warmup:
            rates.append((rate, dt, st))
    value = float(sum(r[2] for r in rates) / sum(r[1] for r in rates))
    line = {
        "impl": "reference", "metric": "ray-steps/s", "value": value, "unit": "ray-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * float(np.mean([r[1] for r in rates])), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": "schwarzschild shadow sweep (2^20 equatorial rays, alpha~U[10,20] deg, r_obs 20M, "
                               "h 0.01, cap 200000) + 64x40 bisections; reference arm: bounded uniform sample "
                               f"of {n} sweep rays per step", "rays_per_step": n},
        "cpu_baseline": {"value": value, "unit": "ray-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{n} rays per step, uniform over the 2^20-ray sweep"},
        "e2e": {"value": value, "unit": "ray-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def pct(v, q):
    return float(np.percentile(np.asarray(v, dtype=np.float64), q)) if len(v) else None


def leg(name, fn, *a, **kw):
    """Run one measurement leg; an exception is reported in the line (and on
    stderr) instead of losing the headline."""
    t0 = time.perf_counter()
    try:
        out = fn(*a, **kw)
    except Exception as e:  # noqa: BLE001 - reported, not hidden
        traceback.print_exc()
        out = {"error": f"{type(e).__name__}: {e}"}
    print(f"[bench] leg {name}: {time.perf_counter() - t0:.1f} s", file=sys.stderr, flush=True)
    return out


class SweepRunner:
    """One step of the headline workload on the GPU: the sweep on stream sa and
    the bisections on stream sb, CUDA events on both. Two schedules. Serial
    (the mixed path's default): the bisection rounds first, alone on the GPU
    (a few ms: each round is as long as its slowest ray takes to settle, and
    alone every ray runs at full speed), then the sweep on every block slot.
    Overlap (the FP64 path's default, where the bisection is the long pole): the
    sweep's persistent grid keeps `reserve` block slots per SM free and the
    bisections run beside it."""

    def __init__(self, lib, torch, h, args, dev):
        self.lib, self.torch, self.h, self.args = lib, torch, h, args
        self.sa, self.sb = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
        self.d_term = torch.empty(N_SWEEP, dtype=torch.int32, device=dev)
        self.d_steps = torch.empty(N_SWEEP, dtype=torch.int64, device=dev)
        self.d_ac = torch.empty(N_BRACKETS, dtype=torch.float64, device=dev)
        self.d_bst = torch.empty(N_BRACKETS, dtype=torch.int64, device=dev)

    def check(self, rc):
        if rc != 0:
            raise RuntimeError(self.lib.geon_last_error().decode())

    def serial(self, precision):
        sched = self.args.schedule
        return precision == 1 if sched == "auto" else sched == "serial"

    def step(self, precision, alpha, lo, hi, r_obs=R_OBS, bisect=True, reserve=None):
        torch, lib = self.torch, self.lib
        n = alpha.numel()
        serial = self.serial(precision) and bisect
        main = torch.cuda.current_stream()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
        ev[0].record(main)
        self.sa.wait_stream(main)
        self.sb.wait_stream(main)
        ev[3].record(self.sb)
        if bisect:
            self.check(lib.geon_shadow_bisect_dev(self.h, r_obs, lo.data_ptr(), hi.data_ptr(), lo.numel(), ITERS,
                                                  STEP, MAX_STEPS, precision, self.d_ac.data_ptr(), None, None,
                                                  self.d_bst.data_ptr(), self.sb.cuda_stream))
        ev[4].record(self.sb)
        if serial:
            self.sa.wait_stream(self.sb)  # the sweep after the bisection rounds, on every slot
        ev[1].record(self.sa)
        lib.geon_set_persistent_reserve_f(0.0 if serial else (self.args.reserve if reserve is None else reserve))
        self.check(lib.geon_shadow_classify_dev(self.h, r_obs, alpha.data_ptr(), n, STEP, MAX_STEPS, precision,
                                                self.d_term.data_ptr(), self.d_steps.data_ptr(),
                                                self.sa.cuda_stream))
        lib.geon_set_persistent_reserve(0)
        ev[2].record(self.sa)
        main.wait_stream(self.sa)
        main.wait_stream(self.sb)
        ev[5].record(main)
        return ev

    def result(self, ev, n, bisect=True):
        self.torch.cuda.synchronize()
        steps = int(self.d_steps[:n].sum().item()) + (int(self.d_bst.sum().item()) if bisect else 0)
        return {"ms": ev[0].elapsed_time(ev[5]), "sweep_ms": ev[1].elapsed_time(ev[2]),
                "bisection_ms": ev[3].elapsed_time(ev[4]), "steps": steps,
                "sweep_steps": int(self.d_steps[:n].sum().item())}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "fp64fast"])
    ap.add_argument("--cpu-rays", type=int, default=4096)
    ap.add_argument("--bisect-rays", type=int, default=BISECT_RAYS,
                    help="speculative bisection width (rays per round over all brackets)")
    ap.add_argument("--schedule", default="auto", choices=["auto", "serial", "overlap"],
                    help="bisections before the sweep (serial: the mixed path's default) or beside it "
                         "(overlap: the FP64 path's default)")
    ap.add_argument("--reserve", type=float, default=RESERVE,
                    help="block slots per SM the sweep leaves free for the bisections (latency vs throughput)")
    ap.add_argument("--fp64-sample", type=int, default=32, help="accuracy and FP64 legs trace every k-th sweep ray")
    ap.add_argument("--fp64-steps", type=int, default=3, help="timed steps of the FP64 latency leg")
    ap.add_argument("--variant", type=int, default=-1,
                    help="mixed equatorial kernel variant (register cap + 3 x block size index); -1: the autotuner's")
    ap.add_argument("--sweep-order", type=int, default=1, help="longest-first claim order of the sweep (1) or not (0)")
    ap.add_argument("--legs", default="all",
                    help="comma list of legs beside the headline (accuracy,fp64,e2e,cpu,config1,config3,config4,"
                         "r30), 'all' or 'none'")
    # small cases for profiling only (they change the workload; never a bench line)
    ap.add_argument("--rays", type=int, default=N_SWEEP, help="profiling: sweep size")
    ap.add_argument("--sweep-only", action="store_true", help="profiling: no bisections")
    ap.add_argument("--escape-radius", type=float, default=SCHW[2], help="profiling: escape radius in M")
    args = ap.parse_args()
    assert args.warmup >= 3, "at least 3 warm-up steps"

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import geon_gb300 as geon
    from geon_gb300 import _ffi, shard
    lib = _ffi.load()
    prec = {"fp64": 0, "mixed": 1, "fp64fast": 3}[args.precision]
    m = geon.Schwarzschild(SCHW[0], SCHW[1], args.escape_radius)
    alpha, lo, hi = rank_workload(rank)
    n_sweep = args.rays
    alpha = alpha[:n_sweep]
    dev = torch.device("cuda", local)
    tuned = geon.autotune.autotune(geon.Schwarzschild(SCHW[0], SCHW[1], 100.0)) if prec == 1 else None
    d_alpha = torch.tensor(alpha, device=dev)
    d_lo = torch.tensor(lo, device=dev)
    d_hi = torch.tensor(hi, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2
    run = SweepRunner(lib, torch, m.handle, args, dev)
    lib.geon_set_bisect_rays_per_round(args.bisect_rays)
    lib.geon_set_sweep_order(args.sweep_order)
    if args.variant >= 0:
        lib.geon_set_mixed_variant(1, 1, args.variant)
    bis = not args.sweep_only

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        run.result(run.step(prec, d_alpha, d_lo, d_hi, bisect=bis), n_sweep, bis)
        flush.zero_()
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = lib.geon_launch_count()
    res = []
    barrier()
    for _ in range(args.steps):
        ev = run.step(prec, d_alpha, d_lo, d_hi, bisect=bis)
        res.append(run.result(ev, n_sweep, bis))
        flush.zero_()  # between timed iterations, outside the events
    barrier()
    launches = lib.geon_launch_count() - launches0
    clocks = sampler.stop()
    times = [r["ms"] for r in res]
    t_total, total_steps = shard_totals(dist, sum(times) / 1e3, sum(r["steps"] for r in res), dev)
    value = total_steps / t_total
    sweep_steps = res[-1]["sweep_steps"]
    ac_run = run.d_ac.cpu().numpy()
    full = n_sweep == N_SWEEP and bis and args.escape_radius == SCHW[2]
    legs = set() if args.legs == "none" or not full else (
        {"accuracy", "fp64", "e2e", "cpu", "config1", "config3", "config4", "r30"} if args.legs == "all"
        else set(args.legs.split(",")))
    extras = {}
    # the plain FP64 path on the same kind of step (every rank: a shard of the job)
    if prec == 1 and "fp64" in legs:
        extras["fp64_path"] = leg("fp64_path", fp64_latency_leg, run, torch, flush, d_alpha, d_lo, d_hi, args,
                                  value, 0, args.fp64_steps)
        extras["fp64fast_path"] = leg("fp64fast_path", fp64_latency_leg, run, torch, flush, d_alpha, d_lo, d_hi,
                                      args, value, 3, 1)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    peak32 = ctypes_peak(lib, 0)
    peak64 = ctypes_peak(lib, 1)
    kernel_s = float(np.mean([r["sweep_ms"] for r in res])) / 1e3
    achieved = ALG_FLOPS_PER_STEP * sweep_steps / kernel_s / 1e12
    peak = peak32 if prec == 1 else peak64
    roofline = {"bound": "fp32 pipe" if prec == 1 else "fp64 pipe", "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak, "traffic": load_traffic(),
                "kernel": "trace_mixed_kernel<Schwarzschild, equatorial, shadow>" if prec == 1 else
                "trace_fp64_kernel<Schwarzschild, equatorial, shadow>",
                "alg_flops_per_ray_step": ALG_FLOPS_PER_STEP,
                "peak_source": "measured in this run: FFMA/DFMA throughput probe (geon_probe_fma_peak); "
                               "MEASURED_PEAKS.json has no FP32/FP64 non-tensor peak",
                "peaks_measured": {"fp32_tflops": peak32, "fp64_tflops": peak64}}
    if "accuracy" in legs:
        extras["accuracy"] = leg("accuracy", accuracy_leg, geon, m, alpha, lo, hi, ac_run, args.fp64_sample)
    if "e2e" in legs:
        extras["e2e"] = leg("e2e", e2e_leg, geon, m, alpha, lo, hi, args.precision, min(args.steps, 10))
    if "cpu" in legs:
        extras["cpu_baseline"] = leg("cpu", cpu_leg, alpha, args.cpu_rays)
    if "config1" in legs:
        extras["config1"] = leg("config1", config1_leg, geon, lib, peak64)
    if "config3" in legs:
        extras["config3"] = leg("config3", config3_leg, geon, lib, 2048, 128, 0, peak32, peak64)
    if "config4" in legs:
        extras["config4"] = leg("config4", config4_leg, geon, 128, peak64)
    if "r30" in legs:
        extras["config2_r30"] = leg("r30", r30_leg, geon, lib, run, torch, flush, dev, prec)
    if "fp64_path" in extras and "ray_steps_per_s" in extras["fp64_path"]:
        extras["mixed_over_fp64"] = value / extras["fp64_path"]["ray_steps_per_s"]

    line = {
        "metric": "ray-steps/s", "value": value, "unit": "ray-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {1: "f32 (mixed: FP32 right-hand side, compensated f32-pair state)", 0: "f64",
                  3: "f64 (fast: fused, reassociated)"}[prec],
        "data": "synthetic (seeded alpha and brackets)",
        "config": {"workload": "schwarzschild shadow sweep: 2^20 equatorial rays alpha~U[10,20] deg + 64 concurrent "
                               "40-iteration bisections, r_obs 20M, h 0.01, cap 200000, escape 1000M",
                   "precision": args.precision, "rays_per_gpu": N_SWEEP, "bisections_per_gpu": N_BRACKETS,
                   "l2": "flushed (256 MB write) between timed steps", "parallelism": f"{world} independent shards",
                   "schedule": ("bisection rounds first, then the sweep on every block slot" if run.serial(prec)
                                else f"bisections beside the sweep, {args.reserve} block slots per SM reserved"),
                   "bisect_rays_per_round": args.bisect_rays,
                   "mixed_kernel_variant": lib.geon_get_mixed_variant(1, 1) if prec == 1 else None,
                   "mixed_block_size": (128, 64, 256)[lib.geon_get_mixed_variant(1, 1) // 3] if prec == 1 else None,
                   "sweep_claim_order": "longest first" if args.sweep_order else "index order",
                   "autotune_rates": None if tuned is None else tuned.get("rates")},
        "latency": {"step_ms_p50": pct(times, 50), "step_ms_p99": pct(times, 99),
                    "bisection_ms_p50": pct([r["bisection_ms"] for r in res], 50),
                    "bisection_ms_p99": pct([r["bisection_ms"] for r in res], 99),
                    "sweep_ms_p50": pct([r["sweep_ms"] for r in res], 50),
                    "sweep_ms_p99": pct([r["sweep_ms"] for r in res], 99)},
        "roofline": roofline,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    if "fp64_path" in extras and "latency" in extras["fp64_path"]:
        line["latency"]["fp64"] = extras["fp64_path"]["latency"]
    line.update(extras)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def fp64_latency_leg(run, torch, flush, d_alpha, d_lo, d_hi, args, value, precision, steps):
    """An FP64 precision on the headline's kind of step: every fp64_sample-th
    sweep ray (the whole sweep would take minutes: GB300 runs FP64 at ~1/60 of
    its FP32 rate) beside all 64 bisections, `steps` device-timed steps."""
    sub = d_alpha[:: max(1, args.fp64_sample)].contiguous()
    out = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        out.append(run.result(run.step(precision, sub, d_lo, d_hi), sub.numel()))
    ms = [o["ms"] for o in out]
    rate = sum(o["steps"] for o in out) / (sum(ms) / 1e3)
    return {"ray_steps_per_s": rate, "unit": "ray-steps/s", "steps": steps, "sweep_rays": int(sub.numel()),
            "latency": {"step_ms_p50": pct(ms, 50), "step_ms_p99": pct(ms, 99),
                        "bisection_ms_p50": pct([o["bisection_ms"] for o in out], 50),
                        "bisection_ms_p99": pct([o["bisection_ms"] for o in out], 99),
                        "sweep_ms_p50": pct([o["sweep_ms"] for o in out], 50),
                        "sweep_ms_p99": pct([o["sweep_ms"] for o in out], 99)},
            "sample": f"every {args.fp64_sample}th sweep ray + the 64 bisections per step, CUDA events",
            "mixed_over_this": value / rate}


def accuracy_leg(geon, m, alpha, lo, hi, ac_run, k):
    """Mixed vs FP64 on a uniform 1/k sample of the sweep, both traced by the
    equatorial entry point with the steppers the sweep uses (the mixed path's
    planar step)."""
    sample = alpha[::k]
    r64 = geon.shadow.trace(m, R_OBS, sample, STEP, MAX_STEPS, precision="fp64")
    rmx = geon.shadow.trace(m, R_OBS, sample, STEP, MAX_STEPS, precision="mixed")
    y0 = geon.shadow.equatorial_ray(m, R_OBS, sample)
    rep = geon.accuracy.class_report(m, y0, STEP, MAX_STEPS, rmx.termination, r64.termination)
    esc = geon.accuracy.clean_escapes(m, r64) & geon.accuracy.clean_escapes(m, rmx)
    d64 = m.asymptotic_direction(r64.final_state[esc])
    dmx = m.asymptotic_direction(rmx.final_state[esc])
    ang = np.arccos(np.clip(np.sum(d64 * dmx, axis=1), -1.0, 1.0))
    ac64, _, _, _ = geon.shadow.bisect(m, R_OBS, lo, hi, ITERS, STEP, MAX_STEPS, precision="fp64")
    acm, _, _, _ = geon.shadow.bisect(m, R_OBS, lo, hi, ITERS, STEP, MAX_STEPS, precision="mixed")
    vs_m, _, _, _ = geon.shadow.bisect(m, R_OBS, 0.0, np.pi / 2 - 1e-3, 60, STEP, MAX_STEPS, precision="mixed")
    rel64 = np.abs(b_of(ac64) - B_C) / B_C
    relm = np.abs(b_of(acm) - B_C) / B_C
    return {
        "sample_rays": int(len(sample)),
        "stepper": "the timed planar equatorial step (geon_shadow_trace)",
        "classes_vs_fp64": rep,
        "class_mismatch_vs_fp64_raw": rep["raw_mismatch"],
        "class_mismatch_vs_arbiter": rep["mismatch_vs_arbiter"],
        "escape_dir_angle_err_rad_max": float(ang.max()) if ang.size else None,
        "escape_dir_angle_err_rad_p50": float(np.median(ang)) if ang.size else None,
        "escape_dir_angle_err_rad_p99": float(np.quantile(ang, 0.99)) if ang.size else None,
        "null_drift_max_escaped_mixed": float(np.max(rmx.null_residual[esc])) if esc.any() else None,
        "null_drift_max_escaped_fp64": float(np.max(r64.null_residual[esc])) if esc.any() else None,
        "escapes_compared": int(esc.sum()),
        "b_c_validate_shadow_bracket_mixed_rel_err": float(abs(b_of(vs_m[0]) - B_C) / B_C),
        "b_c_brackets_within_1e-6_mixed": int(np.sum(relm <= 1e-6)),
        "b_c_brackets_within_1e-6_fp64": int(np.sum(rel64 <= 1e-6)),
        "b_c_rel_err_mixed_p50": float(np.median(relm)),
        "b_c_rel_err_mixed_max": float(relm.max()),
        "b_c_rel_err_fp64_p50": float(np.median(rel64)),
        "b_c_rel_err_fp64_max": float(rel64.max()),
        "b_c_this_run_rel_err_max": float(np.max(np.abs(b_of(ac_run) - B_C) / B_C)),
    }


def e2e_leg(geon, m, alpha, lo, hi, prec_name, reps):
    """The public host API with pinned host buffers (copies inside the timed
    region): sweep and bisections on two host threads, `reps` timed steps
    after one warm-up."""
    import torch
    pa = torch.tensor(alpha).pin_memory().numpy()
    plo = torch.tensor(lo).pin_memory().numpy()
    phi = torch.tensor(hi).pin_memory().numpy()
    res = {}

    def sweep():
        res["sweep"] = geon.shadow.classify(m, R_OBS, pa, STEP, MAX_STEPS, precision=prec_name)

    def bis():
        res["bis"] = geon.shadow.bisect(m, R_OBS, plo, phi, ITERS, STEP, MAX_STEPS, precision=prec_name)

    times, steps = [], []
    for i in range(reps + 1):
        t0 = time.perf_counter()
        th = threading.Thread(target=bis)
        th.start()
        sweep()
        th.join()
        dt = time.perf_counter() - t0
        if i > 0:
            times.append(dt)
            steps.append(int(res["sweep"][1].sum()) + int(res["bis"][3].sum()))
    return {"value": float(sum(steps) / sum(times)), "unit": "ray-steps/s",
            "h2d_bytes_per_step": N_SWEEP * 8 + 2 * N_BRACKETS * 8,
            "d2h_bytes_per_step": N_SWEEP * (4 + 8) + N_BRACKETS * (8 * 3 + 8),
            "steps": reps, "ms_p50": 1e3 * pct(times, 50), "ms_p99": 1e3 * pct(times, 99),
            "ms_min": 1e3 * min(times), "ms_max": 1e3 * max(times),
            "api": "geon_shadow_classify + geon_shadow_bisect (host pointers, two threads)"}


def cpu_leg(alpha, n):
    from oracle import oracle as orc
    threads = orc.hardware_threads()
    rate, dt, st, ns = cpu_sample_rate(orc, alpha, n, threads)
    return {"value": rate, "unit": "ray-steps/s", "cores": threads, "kind": "port",
            "sample": f"{ns} rays uniform over the sweep ({st} ray-steps, {dt:.1f} s)"}


def _wall(fn, reps):
    """Best-of-reps wall time of fn() (host API calls return with results on the host)."""
    best, out = 1e30, None
    for _ in range(reps):
        t0 = time.perf_counter()
        out = fn()
        best = min(best, time.perf_counter() - t0)
    return best, out


def _kernel_trace_ms(geon, m, y0, step, max_steps, precision, reps=2):
    """Device time of geon_trace_dev (the trace kernel alone: states resident in
    HBM, CUDA events on the launching stream); returns (ms, total steps)."""
    import torch
    n = len(y0)
    dy0 = torch.tensor(np.ascontiguousarray(y0), device="cuda")
    term = torch.empty(n, dtype=torch.int32, device="cuda")
    yf = torch.empty((n, 8), dtype=torch.float64, device="cuda")
    st = torch.empty(n, dtype=torch.int64, device="cuda")
    rs = torch.empty(n, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()
    ms = []
    for i in range(reps + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        geon.trace_dev(m, n, dy0.data_ptr(), step, max_steps, term.data_ptr(), yf.data_ptr(), st.data_ptr(),
                       rs.data_ptr(), stream=s.cuda_stream, precision=precision)
        e1.record(s)
        torch.cuda.synchronize()
        if i > 0:
            ms.append(e0.elapsed_time(e1))
    return min(ms), int(st.sum().item())


def config1_leg(geon, lib, peak64):
    """BASELINE config 1: Schwarzschild 256^2, observer r 30M, fov 60, h 0.05,
    cap 20000, escape 100M, stars on; and the reference's CUDA kernel at its
    own escape radius (1000M) beside the FP64 paths there."""
    from oracle import oracle as orc
    obs = [0.0, 30.0, np.pi / 2, 0.0]
    cam = geon.Camera(obs, 60.0, 256, 256)
    m = geon.Schwarzschild(1.0, 1.001, 100.0)
    out = {"workload": "schwarzschild render 256x256, r_obs 30M, fov 60, h 0.05, cap 20000, escape 100M, stars on"}
    res = {}
    for prec in ("fp64", "fp64fast", "mixed"):
        cfg = geon.RenderConfig(precision=prec, show_stars=True)
        geon.render(m, cam, cfg)
        dt, (rgb, st, cls, pst) = _wall(lambda: geon.render(m, cam, cfg, with_classes=True), 3)
        res[prec] = {"ray_steps_per_s": st.total_steps / dt, "ms": 1e3 * dt, "total_steps": st.total_steps,
                     "captured": st.captured, "escaped": st.escaped, "diverged": st.diverged, "cls": cls.ravel()}
    y0 = cam.ray_states(cam.tetrad(m))
    for prec in ("fp64fast", "mixed"):
        res[prec]["classes_vs_fp64"] = geon.accuracy.class_report(m, y0, 0.05, 20000, res[prec]["cls"],
                                                                 res["fp64"]["cls"])
    # the FP64 path against the oracle (the reference's algorithm) on a row sample
    rows = np.arange(0, 256, 16)
    threads = orc.hardware_threads()
    ys = y0.reshape(256, 256, 8)[rows].reshape(-1, 8)
    t0 = time.perf_counter()
    oterm, _, osteps, _ = orc.trace(1, [1.0, 1.001, 100.0], ys, 0.05, 20000, math=orc.LIBM, nthreads=threads)
    dt_cpu = time.perf_counter() - t0
    out["fp64_classes_equal_libm_oracle_rows"] = float(np.mean(res["fp64"]["cls"].reshape(256, 256)[rows].ravel()
                                                               == oterm))
    for r in res.values():
        r.pop("cls")
    out["render"] = res
    # kernel-only FP64_FAST time, for its roofline (FP64 pipe)
    kms, ksteps = _kernel_trace_ms(geon, m, y0, 0.05, 20000, "fp64fast")
    ach = ALG_FLOPS_PER_STEP * ksteps / (kms / 1e3) / 1e12
    out["roofline_fp64fast"] = {"bound": "fp64 pipe", "achieved": ach, "peak": peak64, "unit": "TFLOP/s",
                                "frac": ach / peak64 if peak64 else None, "kernel_ms": kms,
                                "kernel": "trace_fp64fast_kernel<array, trace>",
                                "alg_flops_per_ray_step": ALG_FLOPS_PER_STEP}
    kms64, ksteps64 = _kernel_trace_ms(geon, m, y0, 0.05, 20000, "fp64")
    ach64 = ALG_FLOPS_PER_STEP * ksteps64 / (kms64 / 1e3) / 1e12
    out["roofline_fp64"] = {"bound": "fp64 pipe", "achieved": ach64, "peak": peak64, "unit": "TFLOP/s",
                            "frac": ach64 / peak64 if peak64 else None, "kernel_ms": kms64,
                            "kernel": "trace_fp64_kernel<Schwarzschild, array, trace>"}
    # at the reference CUDA program's escape radius (1000M)
    m1000 = geon.Schwarzschild(1.0, 1.001, 1000.0)
    at1000 = {}
    for prec in ("fp64", "fp64fast"):
        cfg = geon.RenderConfig(precision=prec, show_stars=True)
        geon.render(m1000, cam, cfg)
        dt, (_, st) = _wall(lambda: geon.render(m1000, cam, cfg), 2)
        at1000[prec] = {"ms": 1e3 * dt, "total_steps": st.total_steps, "ray_steps_per_s": st.total_steps / dt,
                        "captured": st.captured, "escaped": st.escaped, "diverged": st.diverged}
    ref = reference_gpu_bar(256, 256, 30.0, 60.0, 0.05, 20000, reps=2)
    at1000["reference_cuda_kernel"] = ref
    if "ms" in ref:
        at1000["fp64fast_speedup_over_reference_kernel"] = ref["ms"] / at1000["fp64fast"]["ms"]
        at1000["fp64_speedup_over_reference_kernel"] = ref["ms"] / at1000["fp64"]["ms"]
    at1000["note"] = ("the reference CUDA program's settings: 256x256 r 30 fov 60 h 0.05 cap 20000, escape fixed at "
                      "1000M; ours through the host render API (wall time, copies included), the reference kernel "
                      "wall time around launch + sync")
    out["escape_1000M"] = at1000
    out["cpu_baseline"] = {"value": float(osteps.sum()) / dt_cpu, "unit": "ray-steps/s", "cores": threads,
                           "kind": "port", "sample": f"every 16th row ({len(ys)} rays, {dt_cpu:.1f} s)"}
    return out


def fd_fallback_counts():
    """Algorithmic FP64 work per RK4 step of the finite-difference fallback
    metrics (Alcubierre, Morris-Thorne), with the operations on structurally
    zero entries removed, as counted by the generator of the sparse
    Christoffel symbols (geon_gb300/csrc/gen_sparse_christoffel.py)."""
    import importlib.util
    path = os.path.join(ROOT, "geon_gb300", "csrc", "gen_sparse_christoffel.py")
    spec = importlib.util.spec_from_file_location("gen_sparse_christoffel", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.op_counts()


def config3_leg(geon, lib, n, row_step, check_agreeing=256, peak32=None, peak64=None):
    """BASELINE config 3: 2048^2 Alcubierre (R 2, thickness 0.125, v 0.5,
    observer x = -10 looking +x) and Morris-Thorne (b0 1, observer l = 10)
    renders, fov 90, h 0.05, cap 20000: mixed on the full images; FP64 (the
    reference's FD-fallback Christoffel symbols) on every row_step-th row; the
    oracle on one row."""
    from oracle import oracle as orc
    cases = {"alcubierre": (geon.Alcubierre(2.0, 0.125, 0.5, 0.0), 2, [2.0, 0.125, 0.5, 0.0],
                            [0.0, -10.0, 0.0, 0.0], -1),
             "morris_thorne": (geon.MorrisThorne(1.0), 3, [1.0], [0.0, 10.0, np.pi / 2, 0.0], 1)}
    out = {"workload": f"exotic renders {n}x{n}: alcubierre (R 2, thickness 0.125, v 0.5) and morris-thorne (b0 1), "
                       "fov 90, h 0.05, cap 20000"}
    threads = orc.hardware_threads()
    for name, (m, kind, params, obs, fwd) in cases.items():
        geon.autotune.autotune(m)
        cam = geon.Camera(obs, 90.0, n, n, forward_sign=fwd)
        cfg = geon.RenderConfig(precision="mixed", show_stars=True)
        geon.render(m, geon.Camera(obs, 90.0, 64, 64, forward_sign=fwd), cfg)
        dt, (_, st) = _wall(lambda: geon.render(m, cam, cfg), 1)
        rows = np.arange(0, n, row_step)
        y0 = cam.ray_states(cam.tetrad(m)).reshape(n, n, 8)[rows].reshape(-1, 8)
        t0 = time.perf_counter()
        r64 = geon.trace(m, y0, 0.05, 20000, precision="fp64")
        dt64 = time.perf_counter() - t0
        rmx = geon.trace(m, y0, 0.05, 20000, precision="mixed")
        # the check of agreeing rays re-traces rays that run to the 20000-step cap
        # at 16 sub-steps per step, one warp's latency through the finite-difference
        # Christoffel symbols (~25 s): the tests run it, the default bench line not
        rep = geon.accuracy.class_report(m, y0, 0.05, 20000, rmx.termination, r64.termination,
                                         check_agreeing=check_agreeing)
        esc = geon.accuracy.clean_escapes(m, r64) & geon.accuracy.clean_escapes(m, rmx)
        d64 = m.asymptotic_direction(r64.final_state[esc])
        dmx = m.asymptotic_direction(rmx.final_state[esc])
        ang = np.arccos(np.clip(np.sum(d64 * dmx, axis=1), -1.0, 1.0)) if esc.any() else None
        yc = y0[:n]  # the first sampled row
        t0 = time.perf_counter()
        _, _, osteps, _ = orc.trace(kind, params, yc, 0.05, 20000, math=orc.LIBM, nthreads=threads)
        dt_cpu = time.perf_counter() - t0
        out[name] = {"mixed_ray_steps_per_s": st.total_steps / dt, "mixed_ms": 1e3 * dt,
                     "mixed_total_steps": st.total_steps,
                     "fp64_ray_steps_per_s": float(r64.steps_taken.sum()) / dt64,
                     "fp64_sample": f"every {row_step}th row ({len(y0)} rays), host API wall time",
                     "mixed_over_fp64": (st.total_steps / dt) / (float(r64.steps_taken.sum()) / dt64),
                     "classes_vs_fp64": rep,
                     "escapes_compared": int(esc.sum()),
                     "escape_dir_err_rad_p50": None if ang is None else float(np.median(ang)),
                     "escape_dir_err_rad_p99": None if ang is None else float(np.quantile(ang, 0.99)),
                     "escape_dir_err_rad_max": None if ang is None else float(ang.max()),
                     "cpu_baseline": {"value": float(osteps.sum()) / dt_cpu, "unit": "ray-steps/s", "cores": threads,
                                      "kind": "port", "sample": f"row 0 ({len(yc)} rays, {dt_cpu:.1f} s)"}}
    counts = fd_fallback_counts()
    for name in cases:
        c, o = counts[name], out[name]
        rays = len(np.arange(0, n, row_step)) * n
        o["roofline_fp64"] = {
            "bound": "fp64 pipe", "alg_flops_per_ray_step": c["flops_per_step"],
            "definition": "the reference's finite-difference fallback (metric/mod.rs:25-69, geodesic.rs:38-59) "
                          "with operations on structurally zero entries removed: "
                          f"{c['ops_per_rhs']} per right-hand side from the sparse Christoffel generator, "
                          f"{c['metric_eval_flops_per_rhs']} for the metric at {c['metric_points_per_rhs']} "
                          f"distinct points, x4, + {104} RK4 combine; not counted: {c['calls_per_step']} per step",
            "achieved": o["fp64_ray_steps_per_s"] * c["flops_per_step"] / 1e12, "unit": "TFLOP/s",
            "sample": f"{rays} rays ({(rays + 127) // 128} blocks of 128 on the GPU), host API wall time"}
        o["roofline_mixed"] = {
            "bound": "fp32 pipe", "alg_flops_per_ray_step": MIXED_CLOSED_FORM_FLOPS_PER_STEP[name],
            "definition": "the mixed path's closed-form right-hand side (metric_analytic.cuh; transcendental "
                          "and division calls not counted) x4 + 104 RK4 combine",
            "achieved": o["mixed_ray_steps_per_s"] * MIXED_CLOSED_FORM_FLOPS_PER_STEP[name] / 1e12,
            "unit": "TFLOP/s"}
        for key, peak in (("roofline_fp64", peak64), ("roofline_mixed", peak32)):
            if peak:
                o[key]["peak"] = peak
                o[key]["frac"] = o[key]["achieved"] / peak
    out["mixed_ray_steps_per_s_both"] = (sum(out[c]["mixed_total_steps"] for c in cases)
                                         / sum(out[c]["mixed_ms"] / 1e3 for c in cases))
    # both images in ONE persistent launch (geon_render_batch): the rays of the
    # two metrics share one work queue; each image must equal its single render
    cfg = geon.RenderConfig(precision="mixed", show_stars=True)
    items = [(m, geon.Camera(obs, 90.0, n, n, forward_sign=fwd), cfg) for m, _, _, obs, fwd in cases.values()]
    singles = [geon.render(m, cam, c, with_classes=True) for m, cam, c in items]
    dt, res = _wall(lambda: geon.render_batch(items), 1)
    steps = sum(r[1].total_steps for r in res)
    out["one_launch_both_images"] = {
        "ray_steps_per_s": steps / dt, "ms": 1e3 * dt, "total_steps": steps,
        "images_equal_single_renders": bool(all(np.array_equal(a[0], b[0]) and np.array_equal(a[2], b[2])
                                                for a, b in zip(res, singles))),
        "api": "geon_render_batch: one trace_multi_mixed_kernel launch over 2 x 2048^2 rays, host wall time"}
    return out


def curvature_cpu_leg(orc, params, pts, threads, budget_s=3.0):
    """The config-4 job per grid point (Einstein tensor + T(k, k) for 16 null
    vectors) on the oracle, on a uniform sample of the grid sized to about
    budget_s each: once with the reference's call graph (Riemann formed again
    inside every curvature.rs call: twice for the Einstein tensor, twice per
    vector for T(k, k)) and once with Riemann formed once per point (the same
    bits). The cost does not depend on the vectors' values, so 16 copies of the
    reference's own k = (1, 1, 0, 0) stand in for them."""
    k = np.tile([[1.0, 1.0, 0.0, 0.0]], (16, 1))
    out = {}
    for name, faithful in (("reference_call_graph", True), ("riemann_once", False)):
        def run(m):
            sub = pts[np.linspace(0, len(pts) - 1, m).astype(np.int64)]
            t0 = time.perf_counter()
            orc.curvature(2, params, sub, "einstein", math=orc.LIBM, faithful=faithful, nthreads=threads)
            orc.nec(2, params, sub, k, math=orc.LIBM, faithful=faithful, nthreads=threads)
            return time.perf_counter() - t0
        m = min(len(pts), 256)
        dt = run(m)
        m = int(min(len(pts), max(m, m * budget_s / max(dt, 1e-6))))
        dt = run(m)
        out[name] = {"value": m / dt, "points": m, "seconds": dt}
    return out


def config4_leg(geon, n, peak64, cpu_budget_s=3.0):
    """BASELINE config 4 (FP64): 128^3 Alcubierre (v_s 0.5, R 2, sigma 8) grid,
    Einstein + T(k, k) for 16 null vectors per point; a 4096-point
    Morris-Thorne line; 1e5 Schwarzschild vacuum points (Ricci scalar)."""
    import torch
    from oracle import oracle as orc
    threads = orc.hardware_threads()
    alc = geon.Alcubierre(2.0, 0.125, 0.5, 0.0)
    lo, hi = (-4.0, -4.0, -4.0), (4.0, 4.0, 4.0)
    geon.curvature.grid(alc, lo, hi, (8, 8, 8), nk=16)
    dt_fresh, (pts, ein, nec, _) = _wall(lambda: geon.curvature.grid(alc, lo, hi, (n, n, n), nk=16), 1)
    # the host API as a caller computing grid after grid uses it: the same
    # caller-owned result arrays each call (fresh arrays add the driver's
    # first-use setup of 537 MB of host memory, dt_fresh)
    ein_h, nec_h = np.empty_like(ein), np.empty_like(nec)
    host_ms = []
    for _ in range(4):
        t0 = time.perf_counter()
        geon.curvature.grid_into(alc, lo, hi, (n, n, n), ein_h, nec_h, nk=16)
        host_ms.append(1e3 * (time.perf_counter() - t0))
    dt = float(np.median(host_ms[1:])) / 1e3
    host_same = bool(np.array_equal(ein_h, ein) and np.array_equal(nec_h, nec))
    del ein_h, nec_h
    sub = np.arange(0, len(pts), max(1, len(pts) // 1024))
    oein = orc.curvature(2, [2.0, 0.125, 0.5, 0.0], pts[sub], "einstein", math=orc.GEON, nthreads=threads)
    bit_exact = bool(np.array_equal(oein.reshape(-1, 16), ein[sub].reshape(-1, 16)))
    oein_libm = orc.curvature(2, [2.0, 0.125, 0.5, 0.0], pts[sub], "einstein", math=orc.LIBM, nthreads=threads)
    bit_exact_libm = bool(np.array_equal(oein_libm.reshape(-1, 16), ein[sub].reshape(-1, 16)))
    cpu = curvature_cpu_leg(orc, [2.0, 0.125, 0.5, 0.0], pts, threads, cpu_budget_s)
    st = torch.cuda.current_stream()
    ein_d = torch.empty(len(pts) * 16, dtype=torch.float64, device="cuda")
    nec_d = torch.empty(len(pts) * 16, dtype=torch.float64, device="cuda")
    launch = lambda: geon.curvature.grid_dev(alc, lo, hi, (n, n, n), ein_d, nec_d, nk=16,  # noqa: E731
                                             stream=st.cuda_stream)
    for _ in range(3):
        launch()
    reps = 5
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(reps):
        launch()  # each launch writes 537 MB of results: more than L2 between launches
    e1.record(st)
    torch.cuda.synchronize()
    kernel_ms = e0.elapsed_time(e1) / reps
    dev_same = bool(np.array_equal(ein_d.cpu().numpy().reshape(-1, 16), ein.reshape(-1, 16))
                    and np.array_equal(nec_d.cpu().numpy().reshape(-1, 16), nec.reshape(-1, 16)))
    del ein_d, nec_d
    ach = CURV_FLOPS_PER_POINT * len(pts) / (kernel_ms / 1e3) / 1e12
    mt = geon.MorrisThorne(1.0)
    dt_mt, (mpts, mein, mnec, _) = _wall(lambda: geon.curvature.grid(mt, (-5, np.pi / 2, 0), (5, np.pi / 2, 0),
                                                                     (4096, 1, 1), nk=16), 2)
    i0 = int(np.argmin(np.abs(mpts[:, 1])))
    g = mt.g(mpts[i0])
    T = geon.curvature.stress_energy(mt, mpts[i0])
    ttt_mixed = float(np.linalg.inv(g)[0, 0] * T[0, 0])  # T^t_t at the point nearest the throat
    t_tt = float(T[0, 0])  # T_tt there, the quantity the reference prints against -1/(8 pi)
    rng = np.random.default_rng(7)
    x = np.stack([np.zeros(100000), rng.uniform(3.0, 50.0, 100000), rng.uniform(0.1, np.pi - 0.1, 100000),
                  rng.uniform(0.0, 2 * np.pi, 100000)], axis=1)
    sch = geon.Schwarzschild(1.0)
    dt_s, rs = _wall(lambda: geon.curvature.ricci_scalar(sch, x), 2)
    return {"workload": f"curvature grid {n}^3 alcubierre (v_s 0.5, R 2, sigma 8) einstein + 16 null T(k,k) per point",
            "points_per_s": len(pts) / dt, "host_api_ms": 1e3 * dt,
            "host_api": "geon_curvature_grid into caller-owned host arrays reused across calls: median of 3 after one "
                        "warm-up, results copied back inside the timed call",
            "host_api_ms_fresh_arrays": 1e3 * dt_fresh, "host_api_same_bits": host_same, "kernel_ms": kernel_ms,
            "kernel_points_per_s": len(pts) / (1e-3 * kernel_ms),
            "roofline": {"bound": "fp64 pipe", "achieved": ach, "peak": peak64, "unit": "TFLOP/s",
                         "frac": ach / peak64 if peak64 else None, "kernel": "curvature_grid_kernel<Alcubierre>",
                         "alg_flops_per_point": CURV_FLOPS_PER_POINT,
                         "hbm_gbs": len(pts) * (16 + 16) * 8 / (kernel_ms / 1e3) / 1e9},
            "device_api_same_bits": dev_same, "bit_exact_vs_oracle_geon_sample": bit_exact,
            "bit_exact_vs_oracle_libm_sample": bit_exact_libm,
            "morris_thorne_line": {"points": 4096, "ms": 1e3 * dt_mt, "points_per_s": 4096 / dt_mt,
                                   "T_tt_nearest_throat": t_tt, "T_t_t_nearest_throat": ttt_mixed,
                                   "l_nearest_throat": float(mpts[i0, 1]),
                                   "minus_1_over_8pi": -1.0 / (8.0 * np.pi)},
            "schwarzschild_vacuum": {"points": 100000, "ms": 1e3 * dt_s, "points_per_s": 1e5 / dt_s,
                                     "max_abs_ricci_scalar": float(np.max(np.abs(rs))),
                                     "median_abs_ricci_scalar": float(np.median(np.abs(rs))),
                                     "p99_abs_ricci_scalar": float(np.quantile(np.abs(rs), 0.99)),
                                     "max_abs_ricci_scalar_theta_within_0.3_of_equator":
                                         float(np.max(np.abs(rs)[np.abs(x[:, 2] - np.pi / 2) < 0.3])),
                                     "note": "the reference's algorithm (finite differences of the analytic "
                                             "Christoffel symbols, h = 1e-5): rounding noise ~1e-12 on the "
                                             "equator, growing as 1/sin^2(theta) toward the sampled theta = 0.1"},
            "cpu_baseline": {"value": cpu["reference_call_graph"]["value"], "unit": "grid-points/s",
                             "cores": threads, "kind": "port",
                             "sample": (f"{cpu['reference_call_graph']['points']} grid points, Einstein + 16 T(k,k) "
                                        f"each, curvature.rs call graph ({cpu['reference_call_graph']['seconds']:.1f}"
                                        " s)"),
                             "riemann_once": cpu["riemann_once"]}}


def r30_leg(geon, lib, run, torch, flush, dev, prec):
    """The headline workload at r_obs = 30M (alpha ~ U[5, 15] deg, brackets
    lo ~ U[9, 9.5], hi ~ U[9.8, 10.3] deg around alpha_c = 9.633 deg): one
    device-timed step, and its accuracy on 1/64 of the sweep."""
    alpha, lo, hi = workload_r30(0x5EED + 30)
    m = geon.Schwarzschild(SCHW[0], SCHW[1], SCHW[2])
    da, dlo, dhi = (torch.tensor(v, device=dev) for v in (alpha, lo, hi))
    run.result(run.step(prec, da, dlo, dhi, r_obs=R_OBS_30), N_SWEEP)
    flush.zero_()
    torch.cuda.synchronize()
    r = run.result(run.step(prec, da, dlo, dhi, r_obs=R_OBS_30), N_SWEEP)
    ac = run.d_ac.cpu().numpy()
    rel = np.abs(b_of(ac, R_OBS_30) - B_C) / B_C
    sample = alpha[::64]
    r64 = geon.shadow.trace(m, R_OBS_30, sample, STEP, MAX_STEPS, precision="fp64")
    rmx = geon.shadow.trace(m, R_OBS_30, sample, STEP, MAX_STEPS, precision="mixed")
    y0 = geon.shadow.equatorial_ray(m, R_OBS_30, sample)
    rep = geon.accuracy.class_report(m, y0, STEP, MAX_STEPS, rmx.termination, r64.termination)
    return {"workload": "schwarzschild shadow sweep at r_obs 30M: 2^20 rays alpha~U[5,15] deg + 64x40 bisections "
                        "from lo~U[9,9.5], hi~U[9.8,10.3] deg, h 0.01, cap 200000, escape 1000M",
            "ray_steps_per_s": r["steps"] / (r["ms"] / 1e3), "ms": r["ms"], "sweep_ms": r["sweep_ms"],
            "bisection_ms": r["bisection_ms"], "b_c_rel_err_max": float(rel.max()),
            "b_c_brackets_within_1e-6": int(np.sum(rel <= 1e-6)), "classes_vs_fp64": rep,
            "sample_rays": int(len(sample))}


def ctypes_peak(lib, fp64):
    import ctypes
    v = ctypes.c_double(0.0)
    rc = lib.geon_probe_fma_peak(fp64, ctypes.byref(v))
    return v.value if rc == 0 else None


def load_traffic():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        d = json.load(open(p))
        return d.get("trace_mixed_shadow_bytes_per_launch")
    except (OSError, ValueError):
        return None


def reference_gpu_bar(width, height, r_obs, fov_deg, step, max_steps, reps=5):
    """The reference's own CUDA kernel (cuda/schwarzschild_render.cu trace_kernel,
    compiled from its source by oracle/ref_cu.py) launched as its main() does:
    16x16 blocks, one pixel per thread, M 1, horizon_pad 1.001, escape 1000M.
    Returns its best-of-reps kernel wall time and termination counts."""
    import ctypes
    from oracle import ref_cu
    if not os.path.exists(ref_cu.CUBIN):
        return {"unavailable": "oracle/_ref cubin not built (needs the reference checkout at build time)"}
    cu = ctypes.CDLL("libcuda.so.1")

    def ok(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: CUresult {rc}")

    ctx = ctypes.c_void_p()
    ok(cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
    if not ctx.value:
        dev = ctypes.c_int()
        ok(cu.cuDeviceGet(ctypes.byref(dev), 0), "cuDeviceGet")
        ok(cu.cuDevicePrimaryCtxRetain(ctypes.byref(ctx), dev), "cuDevicePrimaryCtxRetain")
        ok(cu.cuCtxSetCurrent(ctx), "cuCtxSetCurrent")
    mod, fn = ctypes.c_void_p(), ctypes.c_void_p()
    ok(cu.cuModuleLoad(ctypes.byref(mod), ref_cu.CUBIN.encode()), "cuModuleLoad")
    ok(cu.cuModuleGetFunction(ctypes.byref(fn), mod, ref_cu.KERNEL.encode()), "cuModuleGetFunction")
    n = width * height
    d_term, d_final = ctypes.c_uint64(), ctypes.c_uint64()
    ok(cu.cuMemAlloc_v2(ctypes.byref(d_term), ctypes.c_size_t(n * 4)), "cuMemAlloc")
    ok(cu.cuMemAlloc_v2(ctypes.byref(d_final), ctypes.c_size_t(n * 64)), "cuMemAlloc")
    vals = [ctypes.c_int(width), ctypes.c_int(height), ctypes.c_double(r_obs),
            ctypes.c_double(fov_deg * 3.141592653589793 / 180.0), ctypes.c_double(1.0), ctypes.c_double(step),
            ctypes.c_int(max_steps), ctypes.c_double(1.001), ctypes.c_double(1000.0), d_term, d_final]
    params = (ctypes.c_void_p * len(vals))(*[ctypes.addressof(v) for v in vals])
    gx, gy = (width + 15) // 16, (height + 15) // 16
    best = 1e30
    for _ in range(reps + 1):
        t0 = time.perf_counter()
        ok(cu.cuLaunchKernel(fn, gx, gy, 1, 16, 16, 1, 0, None, params, None), "cuLaunchKernel")
        ok(cu.cuCtxSynchronize(), "cuCtxSynchronize")
        best = min(best, time.perf_counter() - t0)
    term = np.empty(n, dtype=np.int32)
    ok(cu.cuMemcpyDtoH_v2(term.ctypes.data_as(ctypes.c_void_p), d_term, ctypes.c_size_t(n * 4)), "cuMemcpyDtoH")
    cu.cuMemFree_v2(d_term)
    cu.cuMemFree_v2(d_final)
    cu.cuModuleUnload(mod)
    return {"ms": 1e3 * best, "rays_per_s": n / best, "captured": int(np.sum(term == 1)),
            "escaped": int(np.sum(term == 2)), "diverged": int(np.sum(term == 0)),
            "launch": f"{gx}x{gy} blocks of 16x16, best of {reps} after one warm-up, wall time around launch+sync"}


def _emit(workload, value, unit, ms, dtype, extra):
    line = {"metric": unit, "value": value, "unit": unit, "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": dtype, "data": "synthetic (seeded)", "config": {"workload": workload}}
    line.update(extra)
    print(json.dumps(line), flush=True)


def render_main(args):
    """BASELINE config 1 as its own line (config1_leg)."""
    import geon_gb300 as geon
    lib = geon._load()
    out = config1_leg(geon, lib, ctypes_peak(lib, 1))
    mx = out["render"]["mixed"]
    _emit(out["workload"], mx["ray_steps_per_s"], "ray-steps/s", mx["ms"], "f32 (mixed)",
          {"config1": out, "timing": "host API wall time, best of 3, inputs and outputs on the host"})


def exotic_main(args):
    """BASELINE config 3 as its own line (config3_leg)."""
    import geon_gb300 as geon
    lib = geon._load()
    out = config3_leg(geon, lib, args.size, args.row_step, 256, ctypes_peak(lib, 0), ctypes_peak(lib, 1))
    _emit(out["workload"], out["mixed_ray_steps_per_s_both"], "ray-steps/s",
          sum(out[c]["mixed_ms"] for c in ("alcubierre", "morris_thorne")), "f32 (mixed)",
          {"config3": out, "timing": "host API wall time"})


def curvature_main(args):
    """BASELINE config 4 as its own line (config4_leg)."""
    import geon_gb300 as geon
    lib = geon._load()
    out = config4_leg(geon, args.grid, ctypes_peak(lib, 1), cpu_budget_s=8.0)
    _emit(out["workload"], out["points_per_s"], "grid-points/s", out["host_api_ms"], "f64",
          {"config4": out, "timing": "host API wall time (includes the copy of results to the host)"})


SERVE_RES = (128, 256, 512, 1024, 2048)


def serve_requests(n, rate, seed):
    """A seeded request stream: Poisson arrivals (mean `rate`/s); 60% renders
    (metric uniform over the four, square resolution uniform over SERVE_RES,
    camera at radius U[10, 40] looking at the origin, fov U[40, 90] deg),
    30% shadow bisections (one bracket, 32 halvings, 31 rays per round),
    10% curvature slabs of 32^3 points (16 null vectors per point)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    reqs = []
    for i in range(n):
        u = rng.random()
        if u < 0.6:
            kind = int(rng.integers(0, 4))
            res = int(SERVE_RES[rng.integers(0, len(SERVE_RES))])
            r = float(rng.uniform(10.0, 40.0))
            fov = float(rng.uniform(40.0, 90.0))
            reqs.append(("render", float(t[i]), kind, res, r, fov))
        elif u < 0.9:
            reqs.append(("bisect", float(t[i]), float(np.radians(rng.uniform(13.0, 14.0))),
                         float(np.radians(rng.uniform(14.5, 15.5)))))
        else:
            reqs.append(("curvature", float(t[i]), int(rng.integers(0, 4)), int(rng.integers(0, 1 << 62))))
    return reqs


def run_serve_stream(geon, reqs, precision, budget, window_s=None):
    """Submit the stream at its arrival times. With window_s, requests stop
    arriving at window_s and whatever is still queued or running then is
    cancelled (its rays finished so far still count as integrated work); the
    latencies of those requests are censored at the window. Returns the
    server's statistics and the per-request outcome."""
    metrics = {0: geon.Minkowski(), 1: geon.Schwarzschild(1.0, 1.001, 100.0),
               2: geon.Alcubierre(2.0, 0.125, 0.5, 0.0), 3: geon.MorrisThorne(1.0)}
    sch = geon.Schwarzschild(1.0)
    grids = {0: ((-10.0, -10.0, -10.0), (10.0, 10.0, 10.0)), 1: ((3.0, 0.3, 0.0), (10.0, 2.8, 6.0)),
             2: ((-4.0, -4.0, -4.0), (4.0, 4.0, 4.0)), 3: ((-5.0, 0.3, 0.0), (5.0, 2.8, 6.0))}
    jobs, t_sub = [], []
    with geon.Server(budget) as srv:
        t0 = time.perf_counter()
        for q in reqs:
            if window_s is not None and q[1] >= window_s:
                break
            wait = q[1] - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            if q[0] == "render":
                _, _, kind, res, r, fov = q
                if kind in (1, 3):
                    obs, fwd = [0.0, r, np.pi / 2, 0.0], 1
                elif kind == 2:
                    obs, fwd = [0.0, -r, 0.0, 0.0], -1
                else:
                    obs, fwd = [0.0, r, 0.0, 0.0], 1
                cam = geon.Camera(obs, fov, res, res, forward_sign=fwd)
                jobs.append(srv.submit_render(metrics[kind], cam, geon.RenderConfig(show_stars=True),
                                              precision=precision))
            elif q[0] == "bisect":
                jobs.append(srv.submit_bisect(sch, R_OBS, q[2], q[3], iters=32, precision=precision,
                                              rays_per_round=31))
            else:
                lo, hi = grids[q[2]]
                jobs.append(srv.submit_curvature(metrics[q[2]], lo, hi, (32, 32, 32), nk=16, seed=q[3],
                                                 with_einstein=True))
            t_sub.append(time.perf_counter() - t0)
        t_submitted = time.perf_counter() - t0
        cancelled = 0
        if window_s is not None:
            rest = window_s - (time.perf_counter() - t0)
            if rest > 0:
                try:
                    srv.wait_all(timeout=rest)
                except TimeoutError:
                    pass
            t_window = time.perf_counter() - t0
            for j in jobs:
                if j.poll() in (0, 1):
                    j.cancel()
                    cancelled += 1
        srv.wait_all()
        t_all = time.perf_counter() - t0
        st = srv.stats()
        states = [j.poll() for j in jobs]
    st["requests"] = len(jobs)
    st["cancelled_at_window"] = cancelled
    st["submit_wall_s"] = t_submitted
    st["drain_wall_s"] = t_all
    st["window_s"] = window_s
    if window_s is not None:
        # requests unfinished at the window end: their latency is at least
        # (window end - arrival); reported beside the completed ones' percentiles
        cens = [1e3 * (t_window - t) for t, s_ in zip(t_sub, states) if s_ != 2]
        st["censored_latencies"] = len(cens)
        st["censored_latency_min_ms"] = min(cens) if cens else None
        st["censored_latency_p50_ms"] = float(np.median(cens)) if cens else None
        st["t_window_s"] = t_window
    st["failed_ids"] = [j.id for j, s_ in zip(jobs, states) if s_ != 2][:10]
    return st


def serve_summary(st, n_offered_s):
    """Per-precision figures of one served run."""
    wall = st["drain_wall_s"]
    steps = st["ray_steps"] + st.get("ray_steps_unfinished", 0.0)
    return {"ray_steps_per_s": steps / wall, "ray_steps_completed_per_s": st["ray_steps"] / wall,
            "grid_points_per_s": st["grid_points"] / wall,
            "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "by_type": st["by_type"],
            "requests": st["requests"], "completed": st["completed"], "failed": st["failed"],
            "cancelled_at_window": st["cancelled_at_window"],
            "unfinished_latency_lower_bound_min_ms": st.get("censored_latency_min_ms"),
            "unfinished_latency_lower_bound_p50_ms": st.get("censored_latency_p50_ms"),
            "offered_requests_per_s": st["requests"] / n_offered_s,
            "sustained_requests_per_s": st["completed"] / wall,
            "wall_s": wall, "window_s": st["window_s"], "launches": st["launches"]}


def serve_main(args):
    """The serving stream for each precision (the same seeded requests) as one
    JSON line; --rates adds a sweep of arrival rates (mixed) that locates the
    saturation rate: the highest offered rate the server sustains."""
    import torch
    torch.cuda.set_device(0)
    import geon_gb300 as geon
    lib = geon._load()
    for kind_metric in (geon.Schwarzschild(1.0, 1.001, 100.0), geon.Alcubierre(2.0, 0.125, 0.5, 0.0),
                        geon.MorrisThorne(1.0), geon.Minkowski()):
        geon.autotune.autotune(kind_metric)
    reqs = serve_requests(args.requests, args.rate, 0x5E4E)
    window = args.window if args.window > 0 else None
    sampler = ClockSampler(0)
    sampler.start()
    launches0 = lib.geon_launch_count()
    out = {}
    for prec in args.serve_precisions.split(","):
        st = run_serve_stream(geon, reqs, prec, args.budget_gb << 30, window)
        offered_s = min(reqs[st["requests"] - 1][1], window or 1e30) if st["requests"] else 1.0
        out[prec] = serve_summary(st, max(offered_s, 1e-3))
        print(f"serving leg {prec}: " + json.dumps(out[prec]), file=sys.stderr, flush=True)
    sweep = []
    for rate in [float(r) for r in args.rates.split(",") if r]:
        rq = serve_requests(max(4, int(rate * args.sweep_window)), rate, 0x5E4E + int(rate * 1000))
        st = run_serve_stream(geon, rq, "mixed", args.budget_gb << 30, args.sweep_window)
        sm = serve_summary(st, args.sweep_window)
        sm["rate"] = rate
        sweep.append(sm)
        print(f"saturation sweep {rate}/s: " + json.dumps(sm), file=sys.stderr, flush=True)
    launches = lib.geon_launch_count() - launches0
    clocks = sampler.stop()
    n_types = {k: sum(1 for q in reqs if q[0] == k) for k in ("render", "bisect", "curvature")}
    main_prec = args.serve_precisions.split(",")[0]
    line = {"metric": "ray-steps/s", "value": out[main_prec]["ray_steps_per_s"], "unit": "ray-steps/s",
            "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": 1e3 * out[main_prec]["wall_s"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (mixed: FP32 right-hand side, compensated f32-pair state)" if main_prec == "mixed" else "f64",
            "data": "synthetic seeded request stream",
            "config": {"workload": f"serving stream: first {len(reqs)} requests of a Poisson stream, mean "
                                   f"{args.rate}/s ({n_types['render']} renders 128^2-2048^2 over 4 metrics, "
                                   f"{n_types['bisect']} 32-halving bisections, {n_types['curvature']} "
                                   f"32^3 curvature slabs)", "budget_gb": args.budget_gb,
                       "window_s": window,
                       "timing": "host wall clock, first submission to the last request's end"},
            "serving": out, "gpu_launches": int(launches), "clocks": clocks}
    if "mixed" in out and "fp64" in out:
        line["serving"]["mixed_over_fp64_ray_steps"] = out["mixed"]["ray_steps_per_s"] / out["fp64"]["ray_steps_per_s"]
    if sweep:
        ok = [s_ for s_ in sweep if s_["cancelled_at_window"] == 0 and s_["failed"] == 0]
        line["serving"]["saturation_sweep"] = sweep
        line["serving"]["saturation_rate_requests_per_s"] = max((s_["rate"] for s_ in ok), default=None)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    if "--workload" in sys.argv:
        ap = argparse.ArgumentParser()
        ap.add_argument("--workload", choices=["serve", "render", "exotic", "curvature"])
        ap.add_argument("--requests", type=int, default=200)
        ap.add_argument("--rate", type=float, default=200.0)
        ap.add_argument("--budget-gb", type=int, default=64)
        ap.add_argument("--serve-precisions", default="mixed",
                        help="comma list; the fp64 stream of 200 requests runs for tens of minutes")
        ap.add_argument("--window", type=float, default=0.0,
                        help="serve: stop arrivals and cancel what is left after this many seconds (0: drain)")
        ap.add_argument("--rates", default="", help="serve: comma list of arrival rates (mixed) to sweep")
        ap.add_argument("--sweep-window", type=float, default=30.0, help="serve: seconds per swept rate")
        ap.add_argument("--size", type=int, default=2048, help="exotic: image side")
        ap.add_argument("--row-step", type=int, default=16, help="exotic: FP64 traces every k-th row")
        ap.add_argument("--grid", type=int, default=128, help="curvature: grid side")
        ap.add_argument("--gpus", type=int, default=1)
        ap.add_argument("--steps", type=int, default=1)
        ap.add_argument("--warmup", type=int, default=3)
        a = ap.parse_args()
        {"serve": serve_main, "render": render_main, "exotic": exotic_main, "curvature": curvature_main}[a.workload](a)
    else:
        main()
