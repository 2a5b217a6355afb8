"""Benchmark of the GB300 EVP-FFT solver step.

Workload (one GPU): 64^3 periodic-Voronoi RVE with 125 grains, Cu-like FCC
crystal, uniaxial tension along z (lateral stresses zero), 2e-4 strain per
increment, plain FP64.  One step = one whole strain increment: the prelude,
the Green-operator fixed-point iterations until the error norms reach
Err = 1e-5 (or IterMax = 200), the increment end.  Metric: voxel-iterations
per second = sum over steps of (voxels x Green iterations) / time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl voce|reference]
                  [--precision fp64|mixed|mixed_ir|mixed_ir_strict|mixed_nr32]
                  [--config cfg2|cfg3|cfg4|cfg5] [--no-extras]

The default line (cfg2, FP64, N = 1) also carries the metric's other
numerators, each measured in the same run:
  forms    config 2 in every precision form (same increments, same timing),
           with each form's error against the FP64 results;
  batched  config 4: 512 RVEs in one batch, 2 whole increments each, in the
           mixed_ir and mixed_nr32 forms, against the plain FP64 path run one
           RVE at a time;
  served   config 5 sample: 200 Poisson requests at 100 req/s (increments
           scaled, stated in the key), served in both forms and by a plain
           FP64 server that solves one request at a time; p50/p99 latency.

--config cfg3 (256^3, every form vs FP64), cfg4 (batched RVEs), cfg5 (served
requests) run those workloads alone.

--impl reference times the CPU implementation of the same step (the oracle's
C restatement of the reference, bit-identical to the reference build, all
host threads) on the same increments: W untimed, then K whole ones timed.
N > 1 (torchrun): independent replicas, one per GPU, no collective on the
data path; the time is the max over ranks.
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

NR_BYTES_PER_VOXEL = 528     # algorithmic bytes per voxel of one Newton kernel launch
ITER_BYTES_PER_VOXEL = 816   # algorithmic bytes per voxel-iteration (plain FP64)
FLUSH_BYTES = 512 << 20      # > 129 MB L2


def _prec(name):
    from voce_gb300 import capi
    return {"fp64": capi.PREC_FP64, "mixed": capi.PREC_MIXED, "mixed_ir": capi.PREC_MIXED_IR,
            "mixed_ir_strict": capi.PREC_MIXED_IR, "mixed_nr32": capi.PREC_MIXED_NR32}[name]


FORMS = ("fp64", "mixed", "mixed_ir", "mixed_ir_strict", "mixed_nr32")
PREC = {k: (lambda k=k: _prec(k)) for k in FORMS}
# the arithmetic types each form computes in
DTYPE = {"fp64": "f64", "mixed": "f32 spectrum+f64 newton",
         "mixed_ir": "f32 spectrum+f64 newton residual+f32 newton correction",
         "mixed_ir_strict": "f32 spectrum+f64 newton residual+f32 newton correction",
         "mixed_nr32": "f32 spectrum+f32 newton+f64 acceptance"}
FORM_DOC = {"mixed": "FP32 spectrum and Green operator; FP64 Newton (exact Jacobian, chord steps "
                     "near the root), hardening, norms, averages",
            "mixed_ir": "FP32 spectrum and Green operator; Newton: FP32 steps choose the start, "
                        "then every accepted step evaluates the residual and flow rule in FP64 with "
                        "the FP64 stop test, its Jacobian and LDL^T correction in FP32; hardening, "
                        "norms, averages in FP64",
            "mixed_ir_strict": "as mixed_ir without the FP32 start: every Newton step evaluates its "
                               "residual and flow rule in FP64",
            "mixed_nr32": "FP32 spectrum and Green operator; FP32 Newton iterations ended by a "
                          "float-float residual acceptance step (FP32-only while the Green error is "
                          "above 1e-4); FP32 per-voxel error norms"}
# whether the form keeps the Newton residual and stop test, the hardening, the
# averages and the per-voxel convergence norms in FP64 (the precision form's
# specification); mixed_nr32 does not (FP32 Newton, FP32 norms)
FORM_SPEC = {"mixed": True, "mixed_ir": True, "mixed_ir_strict": True, "mixed_nr32": False}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="voce", choices=["voce", "reference"])
    p.add_argument("--precision", default=None, choices=list(FORMS),
                   help="default: fp64 (cfg2), mixed_ir (cfg3, cfg4, cfg5)")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="cfg2: the FP64 line only (no forms / batched / served keys)")
    p.add_argument("--no-cpu", action="store_true", help="cfg2: no CPU baseline sample")
    p.add_argument("--no-tune", action="store_true",
                   help="fixed-budget FFT tiles, no tuning launches (profiler runs: the first "
                        "kernel launches a profiler sees are then the solve's own)")
    p.add_argument("--forms", default="",
                   help="cfg3: comma-separated forms to run (default: all)")
    p.add_argument("--extra-rves", type=int, default=512, help="cfg2 line: RVEs of the batched key")
    p.add_argument("--extra-requests", type=int, default=200,
                   help="cfg2 line: requests of the served key")
    p.add_argument("--extra-rate", type=float, default=100.0,
                   help="cfg2 line: arrival rate of the served key, req/s")
    p.add_argument("--extra-inc-scale", type=float, default=0.025,
                   help="cfg2 line: served increments per request = max(1, round(scale x U{10..80}))")
    p.add_argument("--rves", type=int, default=512, help="cfg4: RVEs in the batch")
    p.add_argument("--edge", type=int, default=256, help="cfg3: grid edge (radix 2/3 only)")
    p.add_argument("--increments", type=int, default=2,
                   help="cfg4: whole increments every RVE runs in the timed batch")
    p.add_argument("--requests", type=int, default=200, help="cfg5: requests in the sample")
    p.add_argument("--rate", type=float, default=100.0, help="cfg5: Poisson arrival rate, req/s")
    p.add_argument("--budget-gb", type=float, default=200.0, help="cfg5: server HBM budget, GB")
    p.add_argument("--active-voxels", type=int, default=8000000,
                   help="cfg5: server active limit, voxels in flight (0: HBM budget alone)")
    p.add_argument("--served-only", action="store_true",
                   help="cfg5: serve the chosen form only (no other form, no plain FP64 server)")
    p.add_argument("--ticks-per-round", type=int, default=8,
                   help="cfg5: batch ticks the server runs between admissions")
    p.add_argument("--quantum", type=int, default=0,
                   help="cfg5: ticks after which a running request may be suspended (0: never)")
    p.add_argument("--inc-scale", type=float, default=0.025,
                   help="cfg5: increments per request = round(scale x U{10..80})")
    p.add_argument("--config", default="cfg2", choices=["cfg2", "cfg3", "cfg4", "cfg5"],
                   help="cfg2: the headline line (64^3, FP64); cfg3: 256^3 plane-strain "
                        "compression, FP64 and mixed side by side with the mixed error")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Group:
    """Host-side barrier and max over ranks (gloo); no GPU collective."""

    def __init__(self, world):
        self.world = world
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if not self.dist:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.dist:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())


def whole_job_rate(grp, local_voxel_iterations: float, local_ms: float):
    """Replicas: the voxel-iterations of all ranks over the slowest rank's
    time.  Returns (voxel-iter/s, max ms, total voxel-iterations)."""
    t_max = grp.max(local_ms)
    vi = grp.sum(local_voxel_iterations)
    return vi / (t_max * 1e-3), t_max, vi


class Clocks:
    """nvidia-smi samples every 200 ms while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            t = [x.strip() for x in line.split(",")]
            if len(t) < 9:
                continue
            try:
                sm.append(float(t[1]))
                smax = float(t[2])
            except ValueError:
                continue
            for n, v in zip(names, t[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_case():
    from voce_gb300 import synth
    return synth.config2(n_steps=100)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


# From the ncu capture of kb_nr<0> (FP64 form) on this workload, summarised in
# profiles/kb_nr_fp64_cfg2_64.md: DRAM bytes read + written by one launch over
# 262144 voxels, and the FP64 flops (FMA = 2) per Newton iteration of a voxel
# and per voxel per launch (instruction counts fitted against the Newton
# iterations of each launch; the capture there checks the fit).
KB_NR_FP64_DRAM_BYTES = 268.9e6
KB_NR_FP64_VOXELS = 262144
KB_NR_FP64_FLOPS_PER_NEWTON = 1127
KB_NR_FP64_FLOPS_PER_VOXEL = 307


# The same for kb_nr<1> (mixed_nr32 form, profiles/kb_nr_nr32_cfg2_64.md) and
# kb_nr<0, 0, 1> (mixed_ir form, profiles/kb_nr_mixed_ir_cfg2_64.md); the mixed
# form's chord-step instance of the FP64 Newton kernel moves the same bytes as
# the FP64 one (profiles/kb_nr_mixed_cfg2_64.md).
KB_NR_NR32_DRAM_BYTES = 280.0e6
KB_NR_IR_DRAM_BYTES = 545.3e6


def profiled_traffic(precision="fp64"):
    """DRAM bytes of one Newton launch at 64^3, from the ncu capture of the
    kernel the form runs."""
    b = {"mixed_nr32": KB_NR_NR32_DRAM_BYTES, "mixed_ir": KB_NR_IR_DRAM_BYTES,
         "mixed_ir_strict": KB_NR_IR_DRAM_BYTES}.get(precision, KB_NR_FP64_DRAM_BYTES)
    return b * (64 ** 3) / KB_NR_FP64_VOXELS


def fp64_flops_per_newton_iteration():
    """FP64 flops (FMA = 2) that kb_nr<0> executes per Newton iteration of
    one voxel and per voxel per launch (profiles/kb_nr_fp64_cfg2_64.md)."""
    return KB_NR_FP64_FLOPS_PER_NEWTON, KB_NR_FP64_FLOPS_PER_VOXEL


CFG2_WORKLOAD = ("64^3 periodic Voronoi, 125 grains, Cu FCC (C11=168.4 GPa), n=20, Voce "
                 "hardening, tension z 1e-3/s, 2e-4 strain per increment (config 2), one whole "
                 "increment per step")


def cfg2_config(nv, iters, precision="fp64"):
    """The workload keys both arms report: the increments a step runs and
    their Green-iteration counts (the same for the FP64 GPU path and the
    CPU reference, which agree iteration for iteration)."""
    return {"workload": CFG2_WORKLOAD, "precision": precision, "voxels": nv,
            "green_iterations": iters}


def _oracle_job(case, threads):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    if not os.path.exists(orc.PORT_LIB):
        orc.build_port()
    d = tempfile.mkdtemp(prefix="cpu_")
    return orc.Job(case.write(d), threads=threads)


def cpu_sample(threads: int, n_incr: int = 2):
    """The oracle (C restatement of the reference) on a bounded sample of
    the workload: its first n_incr whole increments, on `threads` threads."""
    case = make_case()
    j = _oracle_job(case, threads)
    t0 = time.perf_counter()
    j.run(n_incr)
    dt = time.perf_counter() - t0
    n_it = sum(j.increment(k)["iters"] for k in range(n_incr))
    j.close()
    return case.mesh.nvox * n_it / dt, dt, n_it


def run_reference(args, rank, world):
    """--impl reference: the CPU implementation of the same step (the
    oracle's C restatement of the reference, bit-identical to the reference
    build) on all host threads: the same W warm-up increments, then the same K
    whole increments the GPU arm times, each timed alone."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    case = make_case()
    nv = case.mesh.nvox
    j = _oracle_job(case, threads)
    j.run(args.warmup)
    dt = 0.0
    iters = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        j.run(1)
        dt += time.perf_counter() - t0
        iters.append(j.increment(args.warmup + k)["iters"])
    j.close()
    v = nv * sum(iters) / dt
    sample = ("increments %d-%d of the same case, whole (uncapped), after %d untimed ones: "
              "%d Green iterations, %.1f s on %d threads" % (args.warmup + 1, args.warmup + args.steps,
                                                            args.warmup, sum(iters), dt, threads))
    out = {
        "impl": "reference", "metric": "voxel_iterations_per_s", "value": v,
        "unit": "voxel-iter/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": cfg2_config(nv, iters),
        "cpu_baseline": {"value": v, "unit": "voxel-iter/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "voxel-iter/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def _e2e_leg(args, lib, nl, slip, case, prec, grp):
    """The metric through the C ABI from host buffers: voce_rve_create from
    pinned host arrays, then K increments, each followed by the stress and
    strain-rate fields copied to pinned host memory.  It runs first in the
    process, so it pays what a new caller pays (tile tuning, module loading,
    graph construction)."""
    import ctypes as C
    import numpy as np
    from voce_gb300 import capi
    nv = case.mesh.nvox
    eul_b = lib.voce_host_alloc(nv * 24)
    gr_b = lib.voce_host_alloc(nv * 4)
    ph_b = lib.voce_host_alloc(nv * 4)
    out_b = lib.voce_host_alloc(2 * nv * 48)
    eul = np.ctypeslib.as_array((C.c_double * (nv * 3)).from_address(eul_b)).reshape(nv, 3)
    gr = np.ctypeslib.as_array((C.c_int * nv).from_address(gr_b))
    ph = np.ctypeslib.as_array((C.c_int * nv).from_address(ph_b))
    outs = np.ctypeslib.as_array((C.c_double * (2 * nv * 6)).from_address(out_b)).reshape(2, 6 * nv)
    eul[:] = case.mesh.euler_deg
    gr[:] = case.mesh.grain
    ph[:] = case.mesh.phase
    grp.barrier()
    t0 = time.perf_counter()
    re = capi.Rve.create(nl, slip, eul, gr, ph, prec)
    e2e_iters = 0
    for k in range(args.steps):
        re.run(1)
        e2e_iters += re.increment(k)["iters"]
        lib.voce_rve_get_field(re._h, 20, outs[0].ctypes.data_as(C.POINTER(C.c_double)))
        lib.voce_rve_get_field(re._h, 21, outs[1].ctypes.data_as(C.POINTER(C.c_double)))
    re.close()
    t_e2e = time.perf_counter() - t0
    grp.barrier()
    t_e2e = grp.max(t_e2e)
    for b in (eul_b, gr_b, ph_b, out_b):
        lib.voce_host_free(b)
    return {"value": grp.sum(float(nv * e2e_iters)) / t_e2e, "unit": "voxel-iter/s",
            "h2d_bytes_per_step": int(nv * 32 / args.steps),
            "d2h_bytes_per_step": int(2 * 6 * 8 * nv),
            "timed": "create from pinned host mesh (first in the process: tile tuning and "
                     "graph construction included) + %d increments, each followed by the stress "
                     "and strain-rate fields copied to pinned host memory" % args.steps}


def _timed_increments(r, warmup, steps):
    """K increments after W, each timed with CUDA events on the RVE's stream
    after an L2 flush; returns (ms list, Green iterations list, Newton
    iterations summed)."""
    r.run(warmup)
    step_ms, iters, nr = [], [], 0.0
    for k in range(steps):
        r.flush_l2(FLUSH_BYTES)
        step_ms.append(r.run_timed(1))
        inc = r.increment(warmup + k)
        iters.append(inc["iters"])
        nr += inc["nr_iters_total"]
    return step_ms, iters, nr


def run_voce(args, rank, world, grp):
    from voce_gb300 import capi, synth  # noqa: F401
    lib = capi.load()
    args.precision = args.precision or "fp64"
    prec = PREC[args.precision]()
    case = make_case()
    nv = case.mesh.nvox
    d = tempfile.mkdtemp(prefix="bench_")
    nl_path = case.write(d)
    nl = capi.read_namelist(nl_path)
    slip = capi.read_slip(os.path.join(d, "mat.sx"))

    # ---- end-to-end leg through the C ABI, host buffers (first) ---------
    e2e = None if args.no_e2e else _e2e_leg(args, lib, nl, slip, case, prec, grp)

    # ---- device-resident leg: K increments timed with CUDA events --------
    # Each increment runs as one CUDA graph (device-side conditional loop
    # over the Green iterations); events on the RVE's stream bracket it.
    r = capi.Rve.create(nl, slip, case.mesh.euler_deg, case.mesh.grain, case.mesh.phase, prec)
    r.run(args.warmup)
    launches0 = r.kernel_launches
    grp.barrier()
    step_ms = []
    iters = []
    nr_iters = 0.0
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        for k in range(args.steps):
            r.flush_l2(FLUSH_BYTES)
            launches0 += 1        # the flush kernel is not part of the step
            step_ms.append(r.run_timed(1))
            inc = r.increment(args.warmup + k)
            iters.append(inc["iters"])
            nr_iters += inc["nr_iters_total"]
    grp.barrier()
    launches = r.kernel_launches - launches0
    tot_ms = sum(step_ms)
    value, t_max, vox_iters = whole_job_rate(grp, float(nv * sum(iters)), tot_ms)
    fp64_ref = {"incs": [r.increment(k) for k in range(args.warmup + args.steps)],
                "sig": r.field("sig_voigt"), "edot": r.field("edot_voigt"), "iters": iters}

    # ---- per-kernel durations: CUDA events around every launch over the
    # next few increments (host-driven loop, same kernels, same stream) ----
    n_prof = min(args.steps, 5)
    r.set_profiling(True)
    r.reset_kernel_times()
    prof_nr_iters = 0.0
    for k in range(n_prof):
        r.flush_l2(FLUSH_BYTES)
        r.run(1)
        prof_nr_iters += r.increment(args.warmup + args.steps + k)["nr_iters_total"]
    kt = r.kernel_times()
    r.set_profiling(False)
    nr_ms, nr_n = kt["nr"]
    nr_avg_s = nr_ms * 1e-3 / max(nr_n, 1)
    peak, peak_kind = measured_peaks()
    achieved = NR_BYTES_PER_VOXEL * nv / nr_avg_s / 1e9
    fp64_peak = lib.voce_measure_fp64_tflops()
    fpi = fp64_flops_per_newton_iteration() if prec == capi.PREC_FP64 else None
    fp64_ach = ((fpi[0] * prof_nr_iters + fpi[1] * nv * nr_n) / (nr_ms * 1e-3) / 1e12) if fpi else None
    r.close()

    # ---- CPU baseline (rank 0, N=1 only) ---------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, dt, n_it = cpu_sample(threads, 1)
        cpu = {"value": v, "unit": "voxel-iter/s", "cores": threads, "kind": "port",
               "sample": "the first whole increment of the same 64^3 case (%d Green iterations, "
                         "%.1f s on %d threads); --impl reference times the increments this line "
                         "times" % (n_it, dt, threads)}

    # ---- the precision, batched and served forms (N=1 only) ------------
    extras = {}
    if world == 1 and not args.no_extras and args.precision == "fp64":
        extras["forms"] = forms_cfg2(args, nl, slip, case, value, fp64_ref)
        extras["batched"] = cfg4_core(args.extra_rves, args.increments, ("mixed_ir", "mixed_nr32"))
        extras["served"] = cfg5_core(args.extra_requests, args.extra_rate, args.extra_inc_scale,
                                     ("mixed_ir", "mixed_nr32"), plain=True, budget_gb=args.budget_gb,
                                     active_voxels=args.active_voxels, quantum=0,
                                     ticks_per_round=args.ticks_per_round)

    if rank != 0:
        return
    conf = cfg2_config(nv, iters, args.precision)
    conf.update({"l2": "flushed (512 MB write) before every step",
                 "parallelism": "replicas" if world > 1 else "single GPU"})
    out = {
        "metric": "voxel_iterations_per_s", "value": value, "unit": "voxel-iter/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPE[args.precision],
        "data": "synthetic",
        "config": conf,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": profiled_traffic(args.precision),
                     "kernel": "kb_nr", "peak_kind": peak_kind,
                     "algorithmic_bytes_per_voxel": NR_BYTES_PER_VOXEL,
                     "avg_launch_ms": nr_avg_s * 1e3},
        "fp64_roof": {"bound": "fp64", "kernel": "kb_nr", "achieved": fp64_ach,
                      "peak": fp64_peak, "unit": "TFLOP/s",
                      "frac": (fp64_ach / fp64_peak) if fp64_ach else None,
                      "peak_kind": "measured by voce_measure_fp64_tflops in this run"},
        "kernel_timing": "CUDA events around every launch over %d increments after the "
                         "timed ones (host-driven loop)" % n_prof,
        "kernel_ms": {k: v[0] for k, v in kt.items()},
        "kernel_launches_timed": {k: v[1] for k, v in kt.items()},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    out.update(extras)
    print(json.dumps(out), flush=True)


def _rel(x, y):
    import numpy as np
    x = np.asarray(x, float)
    y = np.asarray(y, float)
    return float(np.abs(x - y).max() / np.abs(y).max())


def forms_cfg2(args, nl, slip, case, fp64_value, fp64_ref):
    """Config 2 in every precision form: the same W + K increments as the
    FP64 leg, K of them timed the same way; each form's rate against the FP64
    line's and its error against the FP64 results of the same increments."""
    from voce_gb300 import capi
    lib = capi.load()
    nv = case.mesh.nvox
    out = {}
    for name in ("mixed", "mixed_ir", "mixed_ir_strict", "mixed_nr32"):
        lib.voce_set_ir_predictor(0 if name == "mixed_ir_strict" else 1)
        try:
            r = capi.Rve.create(nl, slip, case.mesh.euler_deg, case.mesh.grain, case.mesh.phase,
                                PREC[name]())
        finally:
            lib.voce_set_ir_predictor(1)
        step_ms, iters, nr = _timed_increments(r, args.warmup, args.steps)
        incs = [r.increment(k) for k in range(args.warmup + args.steps)]
        sig, edot = r.field("sig_voigt"), r.field("edot_voigt")
        r.set_profiling(True)
        r.reset_kernel_times()
        r.run(1)
        n_it = r.increment(args.warmup + args.steps)["iters"]
        kus = {k: round(1e3 * t / n_it, 1) for k, (t, n) in r.kernel_times().items() if n > 0}
        r.close()
        v = nv * sum(iters) / (sum(step_ms) * 1e-3)
        out[name] = {
            "value": v, "over_fp64": v / fp64_value, "ms_per_step": sum(step_ms) / args.steps,
            "arithmetic": FORM_DOC[name], "within_precision_spec": FORM_SPEC[name],
            "newton_iterations_per_voxel_iteration": nr / (nv * sum(iters)),
            "kernel_us_per_iteration": kus,
            "error_vs_fp64": {
                "macro_stress_max_rel": max(_rel(x["sig_avg"], y["sig_avg"])
                                            for x, y in zip(incs, fp64_ref["incs"])),
                "sigma_field_max_rel": _rel(sig, fp64_ref["sig"]),
                "edot_field_max_rel": _rel(edot, fp64_ref["edot"]),
                "green_iterations": [iters, fp64_ref["iters"]]}}
    return out


def run_cfg3(args):
    """256^3 periodic Voronoi (4096 grains), plane-strain compression: the
    same increments in FP64 and in both mixed forms; each mixed form's error
    against FP64 on the macro stress curve and on the fields.  `value` is the
    form --precision names (default mixed_nr32)."""
    import numpy as np
    from voce_gb300 import capi, synth
    chosen = args.precision or "mixed_ir"
    t0 = time.perf_counter()
    # config 3 (synth.config3), its mesh tessellated on the GPU
    case = synth.Case("cfg3_%d" % args.edge, _voronoi_mesh(args.edge, 4096, 3), synth.CU_LIKE,
                      synth.plane_strain_compression(), 0.2, 250)
    t_mesh = time.perf_counter() - t0
    d = tempfile.mkdtemp(prefix="cfg3_")
    synth.write_sx(os.path.join(d, "mat.sx"), case.mat)
    synth.write_namelist(os.path.join(d, "input"), case.mesh.dims, case.mat, case.load,
                         time_step=case.time_step, n_steps=case.n_steps)
    nl = capi.read_namelist(os.path.join(d, "input"))
    slip = capi.read_slip(os.path.join(d, "mat.sx"))
    nv = case.mesh.nvox
    out = {}
    lib = capi.load()
    names = [f for f in args.forms.split(",") if f] if args.forms else list(FORMS)
    if chosen not in names:
        names.append(chosen)
    for name in names:
        lib.voce_set_ir_predictor(0 if name == "mixed_ir_strict" else 1)
        try:
            r = capi.Rve.create(nl, slip, case.mesh.euler_deg, case.mesh.grain, case.mesh.phase,
                                PREC[name]())
        finally:
            lib.voce_set_ir_predictor(1)
        r.run(args.warmup)
        ms, its = 0.0, 0
        for k in range(args.steps):
            r.flush_l2(FLUSH_BYTES)
            ms += r.run_timed(1)
            its += r.increment(args.warmup + k)["iters"]
        incs = [r.increment(k) for k in range(args.warmup + args.steps)]
        out[name] = {"value": nv * its / (ms * 1e-3), "ms": ms, "iters": its,
                     "incs": incs, "sig": r.field("sig_voigt"), "edot": r.field("edot_voigt")}
        # where the time goes: one more increment, host-driven, every launch
        # bracketed by CUDA events (same kernels; after the timed region)
        r.set_profiling(True)
        r.reset_kernel_times()
        r.run(1)
        n_it = r.increment(args.warmup + args.steps)["iters"]
        out[name]["kernel_us_per_iteration"] = {
            k: round(1e3 * t / n_it, 1) for k, (t, n) in r.kernel_times().items() if n > 0}
        r.close()

    def rel(x, y):
        x = np.asarray(x, float)
        y = np.asarray(y, float)
        return float(np.abs(x - y).max() / np.abs(y).max())

    b = out.get("fp64")
    forms = {}
    for name, a in out.items():
        if name == "fp64" or b is None:
            forms[name] = {"value": a["value"], "ms_per_step": a["ms"] / args.steps, "iters": a["iters"],
                           "kernel_us_per_iteration": a["kernel_us_per_iteration"]}
            continue
        forms[name] = {
            "value": a["value"], "ms_per_step": a["ms"] / args.steps, "iters": a["iters"],
            "kernel_us_per_iteration": a["kernel_us_per_iteration"],
            "over_fp64": a["value"] / b["value"], "arithmetic": FORM_DOC[name],
            "within_precision_spec": FORM_SPEC[name],
            "error_vs_fp64": {
                "macro_stress_max_rel": max(rel(x["sig_avg"], y["sig_avg"])
                                            for x, y in zip(a["incs"], b["incs"])),
                "sigma_field_max_rel": rel(a["sig"], b["sig"]),
                "edot_field_max_rel": rel(a["edot"], b["edot"]),
                "green_iterations_vs_fp64": [a["iters"], b["iters"]]}}
    a = out[chosen]
    res = {
        "metric": "voxel_iterations_per_s", "value": a["value"], "unit": "voxel-iter/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": a["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPE[chosen], "data": "synthetic",
        "config": {"workload": "%d^3 periodic Voronoi, 4096 grains, Cu FCC, plane-strain " % args.edge +
                               "compression Lzz=-1e-3/s Lxx=+1e-3/s, 2e-4 per increment "
                               "(config 3), %s form" % chosen, "voxels": nv,
                   "mesh_generation_s": t_mesh, "l2": "flushed before every step"},
        "forms": forms,
    }
    print(json.dumps(res), flush=True)


def _voronoi_mesh(n, n_grains, seed):
    """synth.voronoi_mesh(n, n_grains, seed), with the tessellation computed on
    the GPU (voce_mesh_voronoi; the same mesh, tests/test_gpu_voronoi.py)."""
    import numpy as np
    from voce_gb300 import capi, synth
    rng = np.random.Generator(np.random.PCG64(seed))
    seeds = rng.random((n_grains, 3))
    eul_g = synth.so3_uniform_bunge(rng, n_grains)
    eul, grain, phase = capi.mesh_voronoi((n, n, n), seeds, eul_g)
    return synth.Mesh((n, n, n), eul, grain, phase)


def _loguniform_int(rng, lo, hi):
    import math
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def _rve_inputs(case, d, tag):
    """namelist + .sx for a case (the mesh stays in memory)."""
    from voce_gb300 import capi, synth
    sx = os.path.join(d, "mat.sx")
    if not os.path.exists(sx):
        synth.write_sx(sx, case.mat)
    nlp = os.path.join(d, "input_%s" % tag)
    synth.write_namelist(nlp, case.mesh.dims, case.mat, case.load, time_step=case.time_step,
                         n_steps=case.n_steps, err=case.err, iter_max=case.iter_max)
    return capi.read_namelist(nlp), capi.read_slip(sx)


def _plain_class_throughput(cases_by_edge, d):
    """Plain FP64, one RVE at a time (graph mode): voxel-iter/s per grid edge,
    measured on one increment of one RVE of that edge."""
    from voce_gb300 import capi
    thr = {}
    for edge, case in sorted(cases_by_edge.items()):
        nl, sx = _rve_inputs(case, d, "plain%d" % edge)
        r = capi.Rve.create(nl, sx, case.mesh.euler_deg, case.mesh.grain, case.mesh.phase)
        r.run(1)                                  # warm-up increment (graph build)
        ms = r.run_timed(1)
        its = r.increment(1)["iters"]
        thr[edge] = case.mesh.nvox * its / (ms * 1e-3)
        r.close()
    return thr


def _cfg4_cases(n_rves):
    import numpy as np
    from voce_gb300 import synth
    rng = np.random.Generator(np.random.PCG64(4))
    cases = []
    for i in range(n_rves):
        edge = int(rng.choice([16, 32, 48, 64]))
        grains = _loguniform_int(rng, 8, 512)
        load = synth.random_traceless_load(rng)
        mesh = _voronoi_mesh(edge, grains, 10000 + i)
        cases.append(synth.Case("b%d" % i, mesh, synth.CU_LIKE, load, 0.25, 40))
    return cases


def cfg4_core(n_rves, increments, forms):
    """Batched form (config 4): n_rves RVEs with edges drawn from
    {16,32,48,64}, grains log-uniform 8-512, random traceless loads, 2.5e-4
    per increment, advanced in one batch per form (one launch per phase per
    tick, the tick loop a CUDA graph).  Every RVE runs `increments` whole
    increments; the timed region ends when the last finishes.  Against the
    plain FP64 path run one RVE at a time (per-edge rates measured on a whole
    increment, weighted by the sample's voxels).  Accuracy: one RVE per edge
    through a whole first increment in a batch of each form, against the FP64
    form alone."""
    import numpy as np
    from voce_gb300 import capi
    d = tempfile.mkdtemp(prefix="cfg4_")
    t0 = time.perf_counter()
    cases = _cfg4_cases(n_rves)
    t_gen = time.perf_counter() - t0
    nv_tot = sum(c.mesh.nvox for c in cases)
    inputs = [_rve_inputs(c, d, str(i)) for i, c in enumerate(cases)]

    def create(c, inp, prec):
        return capi.Rve.create(inp[0], inp[1], c.mesh.euler_deg, c.mesh.grain, c.mesh.phase, prec)

    out = {}
    kernel_ms = {}
    for name in forms:
        prec = PREC[name]()
        t0 = time.perf_counter()
        rves = [create(c, inp, prec) for c, inp in zip(cases, inputs)]
        t_setup = time.perf_counter() - t0
        b = capi.Batch(prec)
        for r in rves:
            b.add(r, increments)
        warm = 3
        b.run(max_ticks=warm)                         # warm-up (graph build)
        assert all(r.increments_done == 0 for r in rves)
        t0 = time.perf_counter()
        while b.run(max_ticks=50):
            pass
        t_run = time.perf_counter() - t0
        ticks = b.ticks - warm
        # voxel-iterations of the timed region: every Green iteration of the
        # whole increments, less the warm-up ticks (all RVEs active then)
        vi = sum(r.nv * r.increment(k)["iters"] for r in rves for k in range(increments))
        vi -= warm * nv_tot
        out[name] = {"value": vi / t_run, "seconds": t_run, "ticks": ticks,
                     "ms_per_tick": 1e3 * t_run / ticks, "voxel_iterations": vi,
                     "setup_s": t_setup, "arithmetic": FORM_DOC[name],
                     "within_precision_spec": FORM_SPEC[name],
                     "hbm_gb": sum(capi.footprint(c.mesh.dims, prec) for c in cases) / 1e9}
        b.close()
        if name == forms[0]:
            # per-phase breakdown: ticks of one more increment of every RVE,
            # driven from the host with every launch timed (after the timed
            # region)
            prof_ticks = 5
            with capi.Batch(prec) as bp:
                for r in rves:
                    bp.add(r, 1)
                bp.set_profiling(True)
                bp.run(max_ticks=prof_ticks)
                kernel_ms = {k: ms / prof_ticks for k, (ms, n) in bp.kernel_times().items() if n}
        for r in rves:
            r.close()
    # accuracy: one RVE per edge, a whole first increment, batch vs FP64 alone
    sample = {}
    for c, inp in zip(cases, inputs):
        sample.setdefault(c.mesh.dims[0], (c, inp))
    for name in forms:
        errs = {}
        prec = PREC[name]()
        rves = [create(c, inp, prec) for c, inp in sample.values()]
        with capi.Batch(prec) as b:
            for r in rves:
                b.add(r, 1)
            while b.run(max_ticks=200):
                pass
        for (edge, (c, inp)), r in zip(sample.items(), rves):
            with create(c, inp, capi.PREC_FP64) as rr:
                rr.run(1)
                errs[str(edge)] = _rel(r.increment(0)["sig_avg"], rr.increment(0)["sig_avg"])
            r.close()
        out[name]["first_increment_macro_stress_err_vs_fp64"] = errs
    by_edge = {e: c for e, (c, _) in sample.items()}
    thr = _plain_class_throughput(by_edge, d)
    t_plain = sum(c.mesh.nvox / thr[c.mesh.dims[0]] for c in cases)   # per iteration of all RVEs
    plain = nv_tot / t_plain
    for f in out.values():
        f["batched_over_plain"] = f["value"] / plain
    return {"workload": "batched: %d RVEs, edges U{16,32,48,64}, grains log-U[8,512], random "
                        "traceless loads 1e-3/s, 2.5e-4 per increment (config 4), %d whole "
                        "increments per RVE" % (len(cases), increments),
            "rves": len(cases), "voxels": nv_tot, "mesh_generation_s": t_gen,
            "plain_fp64_one_at_a_time": {"value": plain, "per_edge": thr},
            "forms": out, "kernel_ms_per_tick": {forms[0]: kernel_ms},
            "kernel_timing": "CUDA events around every launch of 5 host-driven ticks of one more "
                             "increment of every RVE, after the timed region"}


def run_cfg4(args):
    """--config cfg4: the batched form alone; `value` is the form --precision
    names (default mixed_ir), the other form beside it."""
    chosen = args.precision or "mixed_ir"
    other = "mixed_nr32" if chosen != "mixed_nr32" else "mixed_ir"
    res = cfg4_core(args.rves, args.increments, (chosen, other))
    a = res["forms"][chosen]
    line = {
        "metric": "voxel_iterations_per_s", "value": a["value"], "unit": "voxel-iter/s", "n_gpus": 1,
        "steps": a["ticks"], "warmup": 3, "ms_per_step": a["ms_per_tick"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[chosen],
        "data": "synthetic",
        "config": {"workload": res["workload"] + ", %s form, one batch tick per step" % chosen,
                   "voxels": res["voxels"],
                   "l2": "inputs larger than L2 (%.1f GB of RVE state)" % a["hbm_gb"]},
        "batched_over_plain": a["batched_over_plain"],
    }
    line.update(res)
    print(json.dumps(line), flush=True)


def cfg5_core(n_requests, rate, inc_scale, forms, plain=True, budget_gb=200.0,
              active_voxels=8000000, quantum=0, ticks_per_round=8):
    """Serving form (config 5): Poisson arrivals of RVE solve requests (edges
    U{16,32,64,128}, grains log-U[8,2048], random traceless loads,
    increments max(1, round(inc_scale x U{10..80}))), served with continuous
    batching in each form, against a plain-FP64 server that solves one
    request at a time, on the same arrival trace."""
    import numpy as np
    from voce_gb300 import capi, synth
    rng = np.random.Generator(np.random.PCG64(5))
    d = tempfile.mkdtemp(prefix="cfg5_")
    reqs = []
    t_arr = 0.0
    t0 = time.perf_counter()
    for i in range(n_requests):
        t_arr += rng.exponential(1.0 / rate)
        edge = int(rng.choice([16, 32, 64, 128]))
        grains = _loguniform_int(rng, 8, 2048)
        load = synth.random_traceless_load(rng)
        inc = max(1, int(round(inc_scale * rng.integers(10, 81))))
        mesh = _voronoi_mesh(edge, min(grains, edge ** 3), 20000 + i)
        c = synth.Case("q%d" % i, mesh, synth.CU_LIKE, load, 0.2, inc)
        nl, sx = _rve_inputs(c, d, str(i))
        reqs.append((t_arr, c, nl, sx, inc))
    t_gen = time.perf_counter() - t0

    def serve(precision, one_at_a_time):
        budget = int(budget_gb * (1 << 30))
        lat, vi, pre = [], 0, 0
        t0 = time.perf_counter()
        if one_at_a_time:
            for (ta, c, nl, sx, inc) in reqs:
                wait = ta - (time.perf_counter() - t0)
                if wait > 0:
                    time.sleep(wait)
                r = capi.Rve.create(nl, sx, c.mesh.euler_deg, c.mesh.grain, c.mesh.phase, precision)
                r.run(inc)
                vi += sum(c.mesh.nvox * r.increment(k)["iters"] for k in range(inc))
                r.field("sig_voigt")
                r.close()
                lat.append((time.perf_counter() - t0) - ta)
            return lat, vi, time.perf_counter() - t0, 0
        with capi.Server(precision, budget, ticks_per_round=ticks_per_round) as s:
            s.set_quantum(quantum)
            s.set_active_limit(active_voxels)
            ids = []
            k = 0
            while True:
                now = time.perf_counter() - t0
                while k < len(reqs) and reqs[k][0] <= now:
                    ta, c, nl, sx, inc = reqs[k]
                    sub_wall = time.perf_counter() - t0
                    ids.append((s.submit(nl, sx, c.mesh.euler_deg, c.mesh.grain, c.mesh.phase, inc),
                                ta, sub_wall))
                    k += 1
                run, que = s.poll()
                if k == len(reqs) and run == 0 and que == 0:
                    break
                if run == 0 and que == 0 and k < len(reqs):
                    time.sleep(max(0.0, reqs[k][0] - (time.perf_counter() - t0)))
            span = time.perf_counter() - t0
            for rid, ta, sub_wall in ids:
                info = s.info(rid)
                assert info.status == capi.REQ_DONE, (rid, info.status, info.error)
                # arrival -> done: time in the server plus the poll delay before submission
                lat.append((info.t_done - info.t_submit) + (sub_wall - ta))
                vi += info.voxel_iterations
                pre += info.preemptions
        return lat, vi, span, pre

    out = {}
    runs = [("served_" + f, PREC[f](), False) for f in forms]
    if plain:
        runs.append(("plain_fp64_one_at_a_time", capi.PREC_FP64, True))
    for name, prec, single in runs:
        lat, vi, span, pre = serve(prec, single)
        out[name] = {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                     "throughput": vi / span, "makespan_s": span, "voxel_iterations": vi}
        if not single:
            out[name].update(preemptions=pre, within_precision_spec=FORM_SPEC[name[7:]])
    b = out.get("plain_fp64_one_at_a_time")
    for name, a in out.items():
        if b is not None and name != "plain_fp64_one_at_a_time":
            a.update(throughput_ratio=a["throughput"] / b["throughput"],
                     p50_ratio=b["p50_s"] / a["p50_s"], p99_ratio=b["p99_s"] / a["p99_s"])
    return {"workload": "serving: %d Poisson requests at %.1f req/s, edges U{16,32,64,128}, grains "
                        "log-U[8,2048], random traceless loads, increments max(1, round(%.3g x "
                        "U{10..80})) (config 5 sample), continuous batching" % (
                            len(reqs), rate, inc_scale),
            "requests": len(reqs), "arrival_rate_per_s": rate, "increment_scale": inc_scale,
            "hbm_budget_gb": budget_gb, "active_limit_voxels": active_voxels,
            "ticks_per_round": ticks_per_round,
            "quantum_ticks": quantum, "request_generation_s": t_gen, "runs": out}


def run_cfg5(args):
    """--config cfg5: the served forms alone; `value` is the form --precision
    names (default mixed_ir)."""
    chosen = args.precision or "mixed_ir"
    forms = (chosen,) if args.served_only else (chosen, "mixed_nr32" if chosen != "mixed_nr32" else "mixed_ir")
    res = cfg5_core(args.requests, args.rate, args.inc_scale, forms, plain=not args.served_only,
                    budget_gb=args.budget_gb, active_voxels=args.active_voxels, quantum=args.quantum,
                    ticks_per_round=args.ticks_per_round)
    a = res["runs"]["served_" + chosen]
    line = {
        "metric": "voxel_iterations_per_s", "value": a["throughput"], "unit": "voxel-iter/s",
        "n_gpus": 1, "steps": res["requests"], "warmup": 0,
        "ms_per_step": 1e3 * a["makespan_s"] / res["requests"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[chosen],
        "data": "synthetic",
        "config": {"workload": res["workload"] + ", %s form" % chosen},
        "throughput_ratio": a.get("throughput_ratio"), "p50_ratio": a.get("p50_ratio"),
        "p99_ratio": a.get("p99_ratio"),
    }
    line.update(res)
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.no_tune and args.impl == "voce":
        from voce_gb300 import capi
        capi.load().voce_set_autotune(0)
    if args.impl == "voce" and args.config in ("cfg3", "cfg4", "cfg5"):
        {"cfg3": run_cfg3, "cfg4": run_cfg4, "cfg5": run_cfg5}[args.config](args)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    grp = Group(world)
    run_voce(args, rank, world, grp)


if __name__ == "__main__":
    main()
