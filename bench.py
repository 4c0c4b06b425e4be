#!/usr/bin/env python3
"""Benchmark: FIRE minimisation of the 200^3 multi-constant lattice with
homeotropic z-walls and a centred homeotropic colloid (L1, L2, L3 =
2.32, 1.0, 0.5), FP64, on GB300.

A step is one FIRE iteration (velocity Verlet + force + FIRE update) over the
whole 8,000,000-site lattice.  `value` is site-steps/s with the state resident
in HBM; `e2e` times the same run through the C ABI from pinned host buffers
(upload of Q0 and site types, K iterations, download of the final Q).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

With N > 1 (torchrun) every rank minimises its own replica of the lattice
(independent solves, no collective on the data path); timing is the max over
ranks.  `--impl reference` times the CPU restatement of the reference's CPU
path (the oracle) on this host's cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time to max|F|<1e-6 & site-steps/s, warm-start+FP32 vs plain FIRE, 1 GB300"
WORKLOAD = dict(L=(200, 200, 200), seed=13371, Ls=(2.32, 1.0, 0.5), W=5.3, walls=(0, 199), sphere=((100.0, 100.0, 100.0), 30.0),
                dt=5e-4)
# algorithmic bytes per site for one launch of each FIRE-iteration kernel (FP64 / FP32 state):
#  predictor: read Q,V,F  write Q,V           = 25 values
#  derivative planes: read Q, types, write 15 = 20 values + 1 B
#  force + kick: read Q, V, types, write F, V = 20 values + 1 B (the 15 derivative planes it also
#                reads are this design's intermediate, 120 / 60 B/site, visible in the measured traffic)
#  control: scalars only
KERNEL_BYTES = {8: [200, 161, 161, 0], 4: [100, 81, 81, 0]}
KERNEL_NAMES = ["fire_predictor", "first_derivatives", "force_kick_reduce", "fire_control"]
# the fused iteration: read Q, V, F, types; write Q, V, F (halo re-reads excluded)
FUSED_BYTES = {8: 241, 4: 121}
# split variants from this index on fuse the predictor into the deep-site kernel
SPLIT_FUSED_FIRST = 7


# FP64 instructions per deep bulk site of the split force + kick (135 DFMA, 15.2 DMUL,
# 22.7 DADD counted by ncu; 106 of them the 25-point form over shared sums)
FP64_OPS_PER_DEEP_SITE = 173


def kernel_roofline(lat, esz, N, peak, peak_kind, tag):
    """Dominant kernel of the FIRE iteration, timed with CUDA events per launch."""
    kms, fused = lat.fire_profile(20)
    tuning = lat.fire_tuning()
    names = list(KERNEL_NAMES)
    nbytes = list(KERNEL_BYTES[esz])
    if fused:
        names[2] = "fire_fused"
        nbytes[2] = FUSED_BYTES[esz]
    elif tuning["path"] == "tiled":
        names[2] = "force_kick_tiled"
    elif tuning["path"] == "split" and tuning["variant"] >= SPLIT_FUSED_FIRST:
        # predictor fused into the deep-site kernel (one buffer set in, the other out);
        # the listed sites' derivative planes and force + kick counted with it
        names[1] = "first_derivatives_listed"
        names[2] = "fire_fused_split"
        nbytes[2] = FUSED_BYTES[esz]
    elif tuning["path"] == "split":
        # deep bulk sites over Q (no derivative planes) + the listed sites; derivative planes only at the list
        names[1] = "first_derivatives_listed"
        names[2] = "force_kick_split"
    dom = int(np.argmax(kms))
    achieved = nbytes[dom] * N / (kms[dom] / 1e3) / 1e9
    out = {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
           "frac": achieved / peak, "peak_source": peak_kind, "traffic": dram_traffic(names[dom], tag, N),
           "kernel_ms": {n: float(x) for n, x in zip(names, kms) if x > 0},
           "algorithmic_bytes_per_site": nbytes[dom], "sites_per_launch": N}
    out["autotuned"] = tuning
    return out


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d["hbm_gbs"], "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
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
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1", "0x1"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def scale_workload(side):
    """The same geometry on a side^3 lattice (walls at 0 and side-1, centred sphere r = 0.15 side)."""
    WORKLOAD["L"] = (side, side, side)
    WORKLOAD["walls"] = (0, side - 1)
    WORKLOAD["sphere"] = ((side / 2.0, side / 2.0, side / 2.0), 0.15 * side)


def workload_name():
    """The FIRE workload's description, from its current side (200 unless --lattice)."""
    w = WORKLOAD
    n = w["L"][0]
    return (f"{n}^3 lattice, homeotropic z-walls (planes {w['walls'][0]} and {w['walls'][1]}) + centred homeotropic "
            f"sphere r={w['sphere'][1]:g}, W={w['W']:g}, L1-L3 = 2.32/1.0/0.5, FIRE dt=5e-4")


def build_workload_host(q, precision=None):
    """Host set-up of the workload through the package's own host helpers."""
    a, b, c, S0 = q.cli_phase_constants()
    w = WORKLOAD
    Q = q.host_random_nematic(w["L"], w["seed"], S0)
    g = q.Geometry(w["L"], Q)
    for plane in w["walls"]:
        g.add_wall(2, plane, q.HOMEOTROPIC, w["W"], S0)
    g.add_sphere(w["sphere"][0], w["sphere"][1], q.HOMEOTROPIC, w["W"], S0)
    return (a, b, c, S0), g


def make_lattice(q, consts, g, precision):
    a, b, c, S0 = consts
    lat = q.Lattice(WORKLOAD["L"], precision)
    lat.set_params(a, b, c, *WORKLOAD["Ls"])
    lat.set_objects(g.objects())
    return lat


# DRAM bytes per launch of each force + kick strategy on the 200^3 workload:
# dram__bytes_read.sum + dram__bytes_write.sum from ncu (--clock-control none).
# The split kernels were captured on the full 200^3 launch (one-pass metrics);
# the older strategies on a 128^3 case, scaled by the number of sites (their
# traffic grows in proportion to the sites they process).
DRAM_BYTES_PER_LAUNCH = {
    ("force_kick_split", "f64"): 1715513856.0,   # 214.4 B/site (161 algorithmic)
    ("force_kick_split", "f32"): 648814080.0,    # 81.1 B/site (81 algorithmic)
    ("fire_fused_split", "f32"): 939452544.0,    # 117.4 B/site (121 algorithmic)
    ("force_kick_reduce", "f64"): 2872800000.0,  # 359.1 B/site
    ("force_kick_tiled", "f32"): 1082400000.0,   # 135.3 B/site
    ("force_kick_reduce", "f32"): 1124800000.0,  # 140.6 B/site
}


def dram_traffic(kernel, precision_tag, sites=8000000):
    """DRAM bytes per launch measured by ncu for this kernel at 200^3, scaled to
    `sites`; None for a kernel without a capture."""
    v = DRAM_BYTES_PER_LAUNCH.get((kernel, precision_tag))
    return None if v is None else v * sites / 8000000.0


def max_over_ranks(ms, device="cuda"):
    """The job's time: the slowest rank's (every rank's timed region is closed
    by a barrier); the value itself when no process group is running."""
    import torch
    dist = torch.distributed
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world, sites, steps, ms):
    """Whole-job site-steps/s: every replica advances its own lattice of
    `sites` sites by `steps` FIRE iterations within the job's time."""
    return world * sites * steps / (ms / 1e3)


def run_ours(args, rank, world):
    import torch
    import __graft_entry__ as ge
    q = ge.load_package()
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    consts, g = build_workload_host(q)
    N = g.Q.shape[0]
    K, W = args.steps, args.warmup
    dist = world > 1

    def barrier():
        if dist:
            torch.distributed.barrier()

    def timed_fire(precision):
        lat = make_lattice(q, consts, g, precision)
        pinned = args.fire_kernel_fp64 if precision == q.FP64 else args.fire_kernel_fp32
        if pinned != "auto":
            lat.set_fire_kernel({"separate": q.FIRE_SEPARATE, "fused": q.FIRE_FUSED, "tiled": q.FIRE_TILED,
                                 "split": q.FIRE_SPLIT}[pinned])
            variant = args.fire_variant_fp64 if precision == q.FP64 else args.fire_variant_fp32
            if variant >= 0:
                lat.set_fire_variant(variant)
        stream = torch.cuda.Stream()
        lat_stream = stream.cuda_stream
        q._check(q.lib().qmin_set_stream(lat._h, lat_stream))
        lat.set_state(g.Q, g.types)
        lat.fire_init(dt=WORKLOAD["dt"])
        lat.fire_run(W)
        torch.cuda.synchronize()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = lat.launches()
        with ClockSampler(dev) as clk:
            torch.cuda.synchronize()
            e0.record(stream)
            r = lat.fire_run(W + K)
            e1.record(stream)
            torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1)
        return lat, r, ms, lat.launches() - l0, clk.summary()

    if args.forms == "fp32":
        lat32, r32, ms32, launches32, _ = timed_fire(q.FP32)
        lat32.close()
        return {"form": "fp32", "value": N * K / (ms32 / 1e3), "ms_per_step": ms32 / K, "forceMax": r32["forceMax"],
                "gpu_launches": launches32}
    # ---- device-resident FP64 run (the headline)
    lat, r, ms, launches, clocks = timed_fire(q.FP64)
    ms_all = [ms]
    ms = max_over_ranks(ms)
    value = job_value(world, N, K, ms)

    # ---- roofline of the dominant kernel (direct launches, CUDA events per kernel)
    import ctypes as C
    peak, peak_kind = measured_peaks()
    roofline = kernel_roofline(lat, 8, N, peak, peak_kind, "f64")
    # whole-iteration view: 241 B/site for the fused ideal (read Q,V,F,types; write Q,V,F)
    it_ms = ms / (K)
    roofline["iteration_achieved_gbs_at_241B"] = 241 * N / (it_ms / 1e3) / 1e9
    if roofline["kernel"] == "force_kick_split":
        # the FP64 force + kick is bound by the FP64 pipe, not by HBM: the same launch
        # against GB300's FP64 instruction rate (2 per SM per cycle, 304 per cycle over
        # the 152 SMs) at the SM clock sampled during the timed region
        mhz = (clocks or {}).get("sm_mhz") or 2070.0
        t = roofline["kernel_ms"]["force_kick_split"] / 1e3
        achieved = FP64_OPS_PER_DEEP_SITE * N / t / 1e9
        peak_ops = 304 * mhz * 1e6 / 1e9
        roofline["fp64_pipe"] = {"ops_per_site": FP64_OPS_PER_DEEP_SITE, "achieved": achieved, "peak": peak_ops,
                                 "unit": "G FP64 instructions/s", "frac": achieved / peak_ops,
                                 "source": "ncu dfma + dmul + dadd per deep site of the FP64 deep-site kernel "
                                           "(128^3 capture); every site counted at the deep-site figure"}
    fire_state = {"forceMax": r["forceMax"], "iterations": r["iterations"]}
    lat.close()
    if args.forms == "fp64":
        return {"form": "fp64", "value": value, "ms_per_step": ms / K, "roofline": roofline, "gpu_launches": launches}

    # ---- end to end through the C ABI from pinned host memory
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(q, consts, g, K, W, barrier, dist)
    return finish(q, args, rank, world, consts, g, N, K, W, timed_fire, value, ms, launches, clocks, roofline,
                  fire_state, r, e2e, peak, C)


def run_e2e(q, consts, g, K, W, barrier, dist):
    """End to end through the C ABI from pinned host memory.  The timed region
    starts from nothing on the device: a fresh handle (qmin_create, the force
    parameters and objects), the upload of Q0 and the site types, the site
    classes and lists built from the types, the FIRE strategy's choice and
    graph capture, K FIRE iterations and the download of the final Q, then
    qmin_destroy.  `value` is such a job in a process that has met this
    problem before (the autotuner's choice is kept per process); `cold_*` the
    same job after qmin_tuning_cache_clear, the autotuner timing its
    candidates inside the job; `warm_handle_*` the job on a handle that
    already holds this geometry (lists, tuned strategy and graphs kept)."""
    import torch
    N = g.Q.shape[0]
    Qh = torch.from_numpy(g.Q).pin_memory()
    Th = torch.from_numpy(g.types).pin_memory()
    Qout = torch.empty_like(Qh).pin_memory()
    stream = torch.cuda.Stream()

    def job(lat=None):
        fresh = lat is None
        if fresh:
            lat = make_lattice(q, consts, g, q.FP64)
            q._check(q.lib().qmin_set_stream(lat._h, stream.cuda_stream))
        lat.set_state_ptr(Qh.data_ptr(), Th.data_ptr())
        lat.fire_init(dt=WORKLOAD["dt"])
        r = lat.fire_run(K)
        lat.get_state_ptr(Qout.data_ptr(), None, None)
        if fresh:
            lat.close()
        return r

    def timed_fresh_job():
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        r = job()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        barrier()
        return r, max_over_ranks(wall * 1e3)

    job()                        # library and kernels loaded, allocator warm
    q.lib().qmin_tuning_cache_clear()
    _, ms_cold = timed_fresh_job()
    r, ms_fresh = timed_fresh_job()
    # the same job on a handle that already holds the geometry
    lat = make_lattice(q, consts, g, q.FP64)
    q._check(q.lib().qmin_set_stream(lat._h, stream.cuda_stream))
    job(lat)
    lat.fire_run(W)
    torch.cuda.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(stream)
    job(lat)
    e1.record(stream)
    torch.cuda.synchronize()
    wall_warm = time.perf_counter() - t0
    barrier()
    lat.close()
    ms_warm = max_over_ranks(max(e0.elapsed_time(e1), wall_warm * 1e3))
    h2d = N * 5 * 8 + N * 4
    d2h = N * 5 * 8
    world = int(os.environ.get("WORLD_SIZE", 1))
    return {"value": job_value(world, N, K, ms_fresh), "unit": "site-steps/s", "h2d_bytes_per_step": h2d / K,
            "d2h_bytes_per_step": d2h / K, "job_ms": ms_fresh, "iterations": r["iterations"],
            "cold_value": job_value(world, N, K, ms_cold), "cold_job_ms": ms_cold,
            "warm_handle_value": job_value(world, N, K, ms_warm), "warm_handle_job_ms": ms_warm,
            "setup_ms": ms_fresh - ms_warm, "cold_setup_ms": ms_cold - ms_warm,
            "note": "per job, wall clock: fresh handle, upload Q0 (AoS f64) + int32 types, site lists, strategy "
                    "choice and graph capture, K FIRE iterations, download final Q, destroy; bytes amortised over "
                    "K. value: the process has tuned this problem before; cold_*: after qmin_tuning_cache_clear; "
                    "warm_handle_*: a handle already holding this geometry"}


def finish(q, args, rank, world, consts, g, N, K, W, timed_fire, value, ms, launches, clocks, roofline, fire_state,
           r, e2e, peak, C):
    """FP32 form on the same input, then the JSON line (rank 0)."""
    # ---- FP32 form (FP32 state/stencils, FP64 reductions) on the same input
    lat32, r32, ms32, _, _ = timed_fire(q.FP32)
    fp32 = {"value": N * K / (ms32 / 1e3), "unit": "site-steps/s", "ms_per_step": ms32 / K,
            "note": "FP32 state and stencils, FP64 reductions; its error against FP64 is reported at convergence "
                    "in time_to_converge (FIRE trajectories of the two precisions decorrelate step by step)"}
    fp32["roofline"] = kernel_roofline(lat32, 4, N, peak, "measured", "f32")
    fp32["roofline"]["iteration_achieved_gbs_at_121B"] = 121 * N / (ms32 / K / 1e3) / 1e9
    lat32.close()
    # the FP32 form's figures as scalars of the headline roofline object too
    roofline["fp32_form_site_steps_per_s"] = fp32["value"]
    roofline["fp32_form_ms_per_step"] = fp32["ms_per_step"]
    roofline["fp32_kernel"] = fp32["roofline"]["kernel"]
    roofline["fp32_kernel_achieved_gbs"] = fp32["roofline"]["achieved"]
    roofline["fp32_kernel_frac"] = fp32["roofline"]["frac"]
    roofline["fp32_iteration_achieved_gbs_at_121B"] = fp32["roofline"]["iteration_achieved_gbs_at_121B"]
    roofline["fp32_iteration_frac_at_121B"] = fp32["roofline"]["iteration_achieved_gbs_at_121B"] / peak

    ttc = None
    if not args.no_configs:
        t64 = time_to_converge(q, consts, g, q.FP64)
        t32 = time_to_converge(q, consts, g, q.FP32)
        t32["E_rel_err_vs_fp64"] = abs(t32["E_per_site"] - t64["E_per_site"]) / abs(t64["E_per_site"])
        ttc = {"rule": "forceMax < 1e-6 (energyMinimizerFIRE forceMax), from the seeded Q0", "fp64": t64,
               "fp32_form": t32, "fp32_speedup": t64["time_s"] / t32["time_s"]}
        if os.path.exists(WARMNET_WEIGHTS):
            ttc["warm_start_fp32"] = warm_start_c2(q, consts, g, t64, t32)

    out = None
    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "site-steps/s", "n_gpus": world, "steps": K, "warmup": W,
               "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f64", "data": "synthetic (seeded random-director Q0, reference geometry builders)",
               "config": {"workload": workload_name() + ", CLI FIRE params",
                          "sites": N, "fire_steps_per_run": K, "precision": "fp64",
                          "l2": "inputs larger than L2 (Q,V,F state = 960 MB)",
                          "parallelism": "replicas" if world > 1 else "single GPU"},
               "clocks": clocks, "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
               "fire_state_after_run": fire_state, "fp32_form": fp32, "time_to_converge": ttc}
        if not args.no_configs:
            out["other_configs"] = {"c1": run_c1(q), "c3": run_c3(q)}
            if os.path.exists(WARMNET_WEIGHTS) and args.c4_test > 0:
                out["other_configs"]["c4"] = run_c4(q, args.c4_test)
    return out


C1_PIN = {"forceMax": 0.0020673379594514331, "E": -0.10040721037532596}  # reference CLI, 50^3, 100 FIRE steps


def run_c1(q):
    """openQmin -i 100 -l 50 --L1 2.32: 50^3 one-constant, 100 FIRE steps, FP64."""
    import torch
    a, b, c, S0 = q.cli_phase_constants()
    L = (50, 50, 50)
    Q = q.host_random_nematic(L, 13371, S0)
    lat = q.Lattice(L, q.FP64)
    lat.set_params(a, b, c, 2.32)
    lat.set_objects([])
    lat.set_state(Q, np.zeros(L[0] * L[1] * L[2], dtype=np.int32))
    lat.fire_init()
    lat.fire_run(3)  # warm-up (tuning, graph capture)
    lat.set_state(Q, np.zeros(L[0] * L[1] * L[2], dtype=np.int32))
    lat.fire_init()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = lat.fire_run(100)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    e, _ = lat.energy()
    lat.close()
    return {"workload": "50^3 one-constant L1=2.32, seed 13371, 100 FIRE steps, FP64 (reference CLI default run)",
            "wall_s": dt, "site_steps_per_s": 125000 * 100 / dt, "forceMax": r["forceMax"], "E_per_site": e,
            "forceMax_rel_err_vs_reference": abs(r["forceMax"] - C1_PIN["forceMax"]) / C1_PIN["forceMax"],
            "E_rel_err_vs_reference": abs(e - C1_PIN["E"]) / abs(C1_PIN["E"])}


def run_c3(q, nsolves=512, max_iterations=30000):
    """512 independent solves, sides U{16..64}, one planar FG sphere each, to forceMax < 1e-6."""
    import ctypes as C
    import importlib
    import torch
    wl = importlib.import_module("qmin_gb300.workloads")
    solves = [wl.c3_solve(s) for s in range(nsolves)]
    sizes = np.array([np.prod(d["L"]) for d in solves], dtype=np.float64)
    out = {"workload": f"{nsolves} solves, sides U{{16..64}}, one degenerate planar sphere each (r U[3, L/4], "
                       "W log-uniform [0.1, 10]), one-constant L1=2.32, seeds 0..511, FIRE to forceMax < 1e-6",
           "total_sites": int(sizes.sum())}
    for prec, tag in ((q.FP64, "fp64"), (q.FP32, "fp32")):
        b = q.Batch([d["L"] for d in solves], prec)
        a, bb, c = solves[0]["consts"]
        b.set_params(a, bb, c, 2.32)
        for k, d in enumerate(solves):
            b.set_solve(k, d["Q"], d["types"], d["objects"])
        b.fire_init(force_cutoff=1e-6)
        its = np.zeros(nsolves, dtype=np.int32)
        fm = np.zeros(nsolves)
        conv = C.c_int()
        torch.cuda.synchronize()
        l0 = b.launches()
        t0 = time.perf_counter()
        rc = q.lib().qmin_batch_fire_run(b._h, max_iterations, q._ip(its), q._dp(fm), C.byref(conv))
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        diverged = [int(k) for k in np.nonzero(~np.isfinite(fm))[0]]
        out[tag] = {"time_to_converge_s": dt, "converged": conv.value, "diverged_solves": diverged,
                    "status": int(rc), "iterations_mean": float(its.mean()), "iterations_max": int(its.max()),
                    "site_steps_per_s": float((sizes * its).sum() / dt), "gpu_launches": b.launches() - l0,
                    "chunk_shape": b.tuning()}
        b.close()
    out["note"] = ("diverged solves follow the reference's own FIRE schedule into overflow (checked against the "
                   "oracle in tests/test_gpu_batch.py)")
    return out


def time_to_converge(q, consts, g, precision, max_iterations=20000, fcut=1e-6, net=None):
    """FIRE from Q0 until forceMax < fcut (the metric's stopping rule), device-resident.
    With `net`, the learned warm start (qmin_warm_start: features, forward,
    write-back) runs first, inside the timed region."""
    import torch
    lat = make_lattice(q, consts, g, precision)
    lat.set_state(g.Q, g.types)
    if net is not None:
        lat.warm_start(net)  # first call outside the timed region
    lat.fire_init(dt=WORKLOAD["dt"], force_cutoff=fcut)
    lat.fire_run(1)  # tuning and graph capture outside the timed region
    lat.set_state(g.Q, g.types)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    t_inf = 0.0
    if net is not None:
        lat.warm_start(net)
        t_inf = time.perf_counter() - t0
    lat.fire_init(dt=WORKLOAD["dt"], force_cutoff=fcut)
    r = lat.fire_run(max_iterations)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    e, _ = lat.energy()
    Qf = lat.get_state()[0] if net is not None else None
    lat.close()
    out = {"time_s": dt, "iterations": r["iterations"], "forceMax": r["forceMax"], "converged": r["forceMax"] < fcut,
           "E_per_site": e, "site_steps_per_s": g.Q.shape[0] * r["iterations"] / dt}
    if net is not None:
        out["inference_s"] = t_inf
        out["final_Q"] = Qf
    return out


# trained on 4096 c4 solves, then fine-tuned on 64^3 crops of c2 and c5 lattices (train_warmstart.py)
WARMNET_WEIGHTS = os.path.join(ROOT, "open-qmin_gb300", "weights", "warmnet_c4_crops.npz")


def warm_start_c2(q, consts, g, t64, t32):
    """Learned warm start + FP32 FIRE on the c2 lattice, judged against the
    plain FP64 run: it counts if forceMax (recomputed in FP64) < 1e-6 and
    |E - E_plain| / |E_plain| <= 1e-4, else the plain FP32 solve is charged on top."""
    import importlib
    ws = importlib.import_module("qmin_gb300.warmstart")
    params = np.load(WARMNET_WEIGHTS)["params"]
    net = q.WarmNet(1, WORKLOAD["L"])
    net.set_params(params)
    w = time_to_converge(q, consts, g, q.FP32, net=net)
    l_net = net.launches()
    net.close()
    sol = {"L": tuple(WORKLOAD["L"]), "consts": tuple(consts[:3]), "Ls": WORKLOAD["Ls"], "objects": g.objects(), "types": g.types, "Q": g.Q}
    fm64, e64 = ws.fp64_check(sol, w.pop("final_Q"))
    rel = abs(e64 - t64["E_per_site"]) / abs(t64["E_per_site"])
    ok = bool(fm64 < 1e-6 and rel <= 1e-4)
    charged = w["time_s"] + (0.0 if ok else t32["time_s"])
    w.update({"forceMax_fp64": fm64, "E_per_site_fp64": e64, "E_rel_vs_plain_fp64": rel,
              "E_lower_than_plain": bool(e64 < t64["E_per_site"]), "protocol_pass": ok,
              "protocol_time_s": charged, "protocol_speedup_vs_plain_fp64": t64["time_s"] / charged,
              "protocol_speedup_vs_plain_fp32": t32["time_s"] / charged,
              "raw_speedup_vs_plain_fp64": t64["time_s"] / w["time_s"], "net_kernel_launches": l_net,
              "weights": os.path.relpath(WARMNET_WEIGHTS, ROOT)})
    return w


def run_warmnet(args):
    """The warm-start net's forward pass on the c2 lattice (or --lattice N^3):
    W untimed passes, then K passes timed with CUDA events on the net's
    stream, for the tcgen05 and the mma.sync convolutions.  FLOPs are the
    convolutions' 2 x rows x cout x taps x cin."""
    import torch
    import __graft_entry__ as ge
    q = ge.load_package()
    consts, g = build_workload_host(q)
    L = WORKLOAD["L"]
    lat = make_lattice(q, consts, g, q.FP32)
    lat.set_state(g.Q, g.types)
    params = np.load(WARMNET_WEIGHTS)["params"]
    flops = 0
    for cin, cout, taps, stride, level in [(16, 32, 27, 1, 0), (32, 48, 27, 2, 0), (48, 64, 27, 2, 1),
                                           (64, 128, 27, 2, 2), (128, 64, 1, 1, 3), (64, 64, 27, 1, 2),
                                           (64, 48, 1, 1, 2), (48, 48, 27, 1, 1), (48, 32, 1, 1, 1),
                                           (32, 32, 27, 1, 0), (32, 16, 1, 1, 0)]:
        out_level = level + (1 if stride == 2 else 0)
        rows = (L[0] >> out_level) * (L[1] >> out_level) * (L[2] >> out_level)
        flops += 2 * rows * cout * taps * cin
    out = {"metric": "warm-start net forward", "unit": "TFLOP/s", "sites": L[0] * L[1] * L[2],
           "conv_gflop_per_forward": flops / 1e9, "config": {"workload": f"{L[0]}^3 c2 geometry, batch 1"}}
    for tc, name in ((1, "tcgen05"), (2, "tcgen05_thread_staged"), (0, "mma_sync")):
        net = q.WarmNet(1, L)
        net.set_params(params)
        net.set_tensor_path(tc)
        st = torch.cuda.Stream()
        net.set_stream(st.cuda_stream)
        lat.warm_start(net)  # features + forward + write-back once
        for _ in range(args.warmup):
            net.forward()
        net.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(args.steps):
            net.forward()
        e1.record(st)
        net.sync()
        ms = e0.elapsed_time(e1) / args.steps
        out[name] = {"ms_per_forward": ms, "tflops": flops / (ms / 1e3) / 1e12}
        net.close()
    out["value"] = out["tcgen05"]["tflops"]
    lat.close()
    return out


def run_kernels(args):
    """One small call of every kernel family, for profilers (ncu -k regex:...):
    on the c2 geometry at side^3 (--lattice), FP64 with the split force + kick
    and FP32 with the fused split iteration (pinned, no tuning): FIRE iterations
    launched one by one, the energy, Adam, Nesterov, L-BFGS, gradient descent,
    defect measures, the allocation-free energy; a one-constant lattice with a
    sphere through the separate kernels and the object forces; 64 batched c3
    solves (persistent launch); the warm-start net's forward, backward and Adam
    step at 64^3.  Prints the CUDA-event time of each call."""
    import ctypes as C
    import importlib
    import torch
    import __graft_entry__ as ge
    q = ge.load_package()
    wl = importlib.import_module("qmin_gb300.workloads")
    consts, g = build_workload_host(q)
    out = {"workload": f"kernel families, {WORKLOAD['L'][0]}^3 c2 geometry", "ms": {}}

    def timed(name, fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        r = fn()
        e1.record()
        torch.cuda.synchronize()
        out["ms"][name] = e0.elapsed_time(e1)
        return r

    fams = set(args.families.split(","))
    for prec, tag, variant in ((q.FP64, "fp64", 1), (q.FP32, "fp32", 9)):
        if tag not in fams:
            continue
        lat = make_lattice(q, consts, g, prec)
        lat.set_fire_kernel(q.FIRE_SPLIT)
        lat.set_fire_variant(variant)
        # single launches first, then the iterative runs (graphs of 16 iterations)
        timed(tag + " set_state", lambda: lat.set_state(g.Q, g.types))
        timed(tag + " energy", lambda: lat.energy())
        timed(tag + " defects", lambda: lat.defect_measures(0))
        timed(tag + " gd 2", lambda: lat.gd_run(2))
        if prec == q.FP64:
            n = g.Q.shape[0]
            Qd = torch.from_numpy(np.ascontiguousarray(g.Q.T)).cuda()
            td = torch.from_numpy(g.types.astype(np.int8)).cuda()
            res = torch.zeros(6, dtype=torch.float64, device="cuda")
            fn = q.lib().qmin_energy_noalloc
            fn.argtypes = [C.c_void_p] * 3 + [C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p]
            fn.restype = C.c_int
            a, b, c, _S0 = consts
            prm = q.LdgParams()
            prm.A, prm.B, prm.C, prm.L1, prm.L2, prm.L3 = a, b, c, *WORKLOAD["Ls"]
            prm.multi_constant = 1
            objs = g.objects()
            oa = (q.Object * len(objs))()
            for k, (kind, W, S0) in enumerate(objs):
                oa[k].kind, oa[k].W, oa[k].S0 = kind, W, S0
            desc = q.LatticeDesc(*WORKLOAD["L"], q.FP64, 0)
            if n <= 8388608:
                timed("energy_noalloc", lambda: fn(C.byref(desc), C.byref(prm), oa, len(objs), Qd.data_ptr(), n,
                                                   td.data_ptr(), res.data_ptr(), None))
        lat.fire_init(dt=WORKLOAD["dt"])
        timed(tag + " fire_run 3", lambda: lat.fire_run(3))
        timed(tag + " fire_profile 2", lambda: lat.fire_profile(2))
        timed(tag + " adam 2", lambda: lat.adam_run(2))
        timed(tag + " nesterov 2", lambda: lat.nesterov_run(2))
        timed(tag + " lbfgs 2", lambda: lat.lbfgs_run(2))
        lat.close()
    s1 = wl.c3_solve(3, 64, 64)
    a, b, c = s1["consts"]
    if "onec" in fams:
        # one-constant lattice with a sphere: separate kernels, object forces
        lat = q.Lattice(s1["L"], q.FP32)
        lat.set_params(a, b, c, 2.32)
        lat.set_objects(s1["objects"])
        lat.set_state(s1["Q"], s1["types"])
        lat.set_fire_kernel(q.FIRE_SEPARATE)
        lat.fire_init()
        timed("one-constant fire_profile 2", lambda: lat.fire_profile(2))
        timed("object forces", lambda: lat.object_forces())
        lat.close()
    if "batch" in fams:
        # batched solves
        solves = [wl.c3_solve(k) for k in range(64)]
        bt = q.Batch([d["L"] for d in solves], q.FP32)
        bt.set_params(a, b, c, 2.32)
        for k, d in enumerate(solves):
            bt.set_solve(k, d["Q"], d["types"], d["objects"])
        bt.fire_init()
        timed("batch fire_run 10", lambda: bt.fire_run(10))
        bt.close()
    if "batchmc" in fams:
        # batched multi-constant solves: 16 c4 solves (64^3, walls + sphere, L1-L3), FP32
        c4s = [wl.c4_solve(100000 + k) for k in range(16)]
        bt = q.Batch([d["L"] for d in c4s], q.FP32)
        a4, b4, cc4 = c4s[0]["consts"]
        bt.set_params(a4, b4, cc4, *c4s[0]["Ls"])
        for k, d in enumerate(c4s):
            bt.set_solve(k, d["Q"], d["types"], d["objects"])
        bt.fire_init()
        timed("batch multi-constant fire_run 10", lambda: bt.fire_run(10))
        bt.close()
    if "net" not in fams:
        return out
    # warm-start net: forward, backward, Adam at 64^3
    s4 = wl.c4_solve(7)
    net = q.WarmNet(1, s4["L"], train=True)
    net.set_params(q.warmnet_init_params(1))
    qd = torch.from_numpy(np.ascontiguousarray(s4["Q"].T)).cuda()
    tdv = torch.from_numpy(s4["types"].astype(np.int8)).cuda()
    net.features(0, qd.data_ptr(), q.FP64, s4["Q"].shape[0], tdv.data_ptr(), s4["objects"])
    tgt = torch.zeros((1, s4["Q"].shape[0], 5), dtype=torch.float32, device="cuda")
    timed("net forward", lambda: (net.forward(), net.sync()))
    timed("net backward", lambda: (net.backward(tgt.data_ptr()), net.sync()))
    timed("net adam", lambda: (net.adam_step(1e-4), net.sync()))
    net.close()
    return out


def run_c4(q, ntest=64):
    """The learned warm start on c4 test solves (64^3, seeds 100000..), judged by the protocol."""
    import importlib
    wl = importlib.import_module("qmin_gb300.workloads")
    ws = importlib.import_module("qmin_gb300.warmstart")
    params = np.load(WARMNET_WEIGHTS)["params"]
    test = [wl.c4_solve(100000 + k) for k in range(ntest)]
    res = ws.evaluate(params, test, log=lambda *a: None)
    res["failed"] = [int(k) for k in res["failed"]]
    res["workload"] = (f"{ntest} c4 test solves: 64^3, homeotropic z-walls, one homeotropic sphere (r U[6.4, 12.8], "
                       "W log-uniform [1, 10]), L1-L3 = 2.32/1.0/0.5, seeds 100000.., to forceMax < 1e-6")
    res["speedup_vs_plain_fp64"] = res["plain_fp64_seconds"] / res["warm_total_seconds"]
    res["speedup_vs_plain_fp32"] = res["plain_fp32_seconds"] / res["warm_total_seconds"]
    return res


def cpu_baseline(sample_iters=2, threads=1):
    """The oracle (CPU restatement of the reference's CPU path) on a bounded
    sample of the same workload: `sample_iters` FIRE iterations of the 200^3
    lattice, timed with wall clock around the FIRE loop.  Returns the baseline
    record, the oracle's FIRE result and its final Q."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import qmin_oracle as qo
    qo.build()
    used = qo.set_threads(threads)
    w = WORKLOAD
    s = qo.System(w["L"], Ls=w["Ls"] + (0.0,))
    s.random_nematic(w["seed"])
    for plane in w["walls"]:
        s.add_wall(2, plane, 0, w["W"])
    s.add_sphere(w["sphere"][0], w["sphere"][1], 0, w["W"])
    t0 = time.perf_counter()
    r = s.fire(sample_iters, dt=w["dt"])
    dt = time.perf_counter() - t0
    # minimize() evaluates the force once on entry: count it as part of the sample's work
    value = s.N * sample_iters / dt
    return {"value": value, "unit": "site-steps/s", "cores": used, "kind": "port",
            "sample": f"{sample_iters} FIRE iterations (+1 entry force evaluation) of the 200^3 workload, "
                      f"{used} thread(s); oracle = C restatement of the reference CPU path"}, r, s.Q


def c2_parity(q, iters, oracle_result, oracle_Q):
    """The headline workload's FP64 FIRE run on the GPU (autotuned strategy)
    after the same `iters` iterations as the oracle's sample: relative error of
    forceMax, and normwise relative error of Q."""
    consts, g = build_workload_host(q)
    lat = make_lattice(q, consts, g, q.FP64)
    lat.set_state(g.Q, g.types)
    lat.fire_init(dt=WORKLOAD["dt"])
    r = lat.fire_run(iters)
    Q = lat.get_state()[0]
    lat.close()
    fo = oracle_result["forceMax"]
    return {"parity_iterations": r["iterations"], "parity_forceMax_gpu": r["forceMax"], "parity_forceMax_oracle": fo,
            "parity_forceMax_rel_err": abs(r["forceMax"] - fo) / fo,
            "parity_Q_rel_err": float(np.abs(Q - oracle_Q).max() / np.abs(oracle_Q).max())}


def run_reference(args):
    """--impl reference: the reference's CPU path (its C restatement) on all host cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import qmin_oracle as qo
    qo.build()
    threads = os.cpu_count() or 1
    used = qo.set_threads(threads)
    w = WORKLOAD
    s = qo.System(w["L"], Ls=w["Ls"] + (0.0,))
    s.random_nematic(w["seed"])
    for plane in w["walls"]:
        s.add_wall(2, plane, 0, w["W"])
    s.add_sphere(w["sphere"][0], w["sphere"][1], 0, w["W"])
    V = np.zeros((s.N, 5))
    # warm-up: one iteration, then time up to K iterations within a bounded budget
    fp = qo.FireParams(w["dt"], 0.99, 100 * w["dt"], 1.1, 0.95, 0.9, 0.0, 1e-12, 4)
    st = qo.FireState()
    lib = qo.lib()
    lib.qo_fire_init(qo.C.byref(fp), qo.C.byref(st))
    F = np.zeros((s.N, 5))
    import ctypes as C
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
    lib.qo_fire(C.byref(s.p), dp(s.Q), dp(V), dp(F), ip(s.types), s.objs, C.byref(fp), max(args.warmup, 1),
                C.byref(st), None)
    budget = 90.0
    done, t0 = 0, time.perf_counter()
    while done < args.steps and time.perf_counter() - t0 < budget:
        target = st.iterations + 1
        lib.qo_fire(C.byref(s.p), dp(s.Q), dp(V), dp(F), ip(s.types), s.objs, C.byref(fp), target, C.byref(st), None)
        done += 1
    el = time.perf_counter() - t0
    value = s.N * done / el
    cpu = {"value": value, "unit": "site-steps/s", "cores": used, "kind": "port",
           "sample": f"{done} FIRE iterations of the {w['L'][0]}^3 workload (each with the minimize() entry force "
                     f"evaluation), {used} OpenMP threads, wall-clock bounded to {budget:.0f} s"}
    return {"metric": METRIC, "value": value, "unit": "site-steps/s", "n_gpus": 0, "steps": done,
            "warmup": max(args.warmup, 1), "ms_per_step": el / max(done, 1) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_name() + ", CLI FIRE params", "sites": s.N},
            "impl": "reference", "cpu_baseline": cpu,
            "e2e": {"value": value, "unit": "site-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_c5(args):
    """400^3, 8 random homeotropic spheres, L1-L3, uniform E field along z:
    plain FP64 FIRE and the FP32 form to forceMax < 1e-6, then Adam and L-BFGS
    (the reference's default parameters, FP32 form) on the same input."""
    import importlib
    import torch
    import __graft_entry__ as ge
    q = ge.load_package()
    wl = importlib.import_module("qmin_gb300.workloads")
    d = wl.c5_lattice(args.lattice if args.lattice != 200 else 400)
    N = d["Q"].shape[0]
    a, b, c = d["consts"]
    out = {"workload": f"{d['L'][0]}^3, {len(d['spheres'])} random homeotropic spheres r U[10,25] W=5.3, "
                       "L1-L3 = 2.32/1.0/0.5, uniform E = (0, 0, 0.5), eps = eps0 = 1, deps = 0.5, seed 13371",
           "sites": N, "spheres": d["spheres"]}

    def lattice(prec):
        lat = q.Lattice(d["L"], prec)
        lat.set_params(a, b, c, *d["Ls"], E=d["E"])
        lat.set_objects(d["objects"])
        lat.set_state(d["Q"], d["types"])
        return lat

    for prec, tag in ((q.FP64, "fire_fp64"), (q.FP32, "fire_fp32")):
        lat = lattice(prec)
        lat.fire_init(force_cutoff=1e-6)
        lat.fire_run(1)
        lat.set_state(d["Q"], d["types"])
        lat.fire_init(force_cutoff=1e-6)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = lat.fire_run(args.c5_max_iterations)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        e, comps = lat.energy()
        out[tag] = {"time_s": dt, "iterations": r["iterations"], "forceMax": r["forceMax"],
                    "converged": r["forceMax"] < 1e-6, "E_per_site": e, "site_steps_per_s": N * r["iterations"] / dt}
        lat.close()
    if os.path.exists(WARMNET_WEIGHTS):
        # learned warm start (net trained on c4 at 64^3, run on the whole 400^3 lattice) + FP32 FIRE
        ws = importlib.import_module("qmin_gb300.warmstart")
        net = q.WarmNet(1, d["L"])
        net.set_params(np.load(WARMNET_WEIGHTS)["params"])
        lat = lattice(q.FP32)
        lat.warm_start(net)  # first call outside the timed region
        lat.fire_init(force_cutoff=1e-6)
        lat.fire_run(1)
        lat.set_state(d["Q"], d["types"])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lat.warm_start(net)
        t_inf = time.perf_counter() - t0
        lat.fire_init(force_cutoff=1e-6)
        r = lat.fire_run(args.c5_max_iterations)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        Qf = lat.get_state()[0]
        lat.close()
        net.close()
        fm64, e64 = ws.fp64_check(d, Qf)
        ep = out["fire_fp64"]["E_per_site"]
        rel = abs(e64 - ep) / abs(ep)
        ok = bool(fm64 < 1e-6 and rel <= 1e-4)
        out["warm_start_fp32"] = {"time_s": dt, "inference_s": t_inf, "iterations": r["iterations"],
                                  "forceMax_fp64": fm64, "E_per_site_fp64": e64, "E_rel_vs_plain_fp64": rel,
                                  "E_lower_than_plain": bool(e64 < ep), "protocol_pass": ok,
                                  "protocol_time_s": dt + (0.0 if ok else out["fire_fp32"]["time_s"]),
                                  "weights": os.path.relpath(WARMNET_WEIGHTS, ROOT)}
    for name, prec in (() if args.c5_fire_only else (("adam", q.FP32), ("lbfgs", q.FP32), ("lbfgs", q.FP64))):
        tag = name + ("_fp32" if prec == q.FP32 else "_fp64")
        lat = lattice(prec)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        try:
            if name == "adam":
                r = lat.adam_run(args.c5_max_iterations, force_cutoff=1e-6)
            else:
                r = lat.lbfgs_run(args.c5_max_iterations, force_cutoff=1e-6)
        except q.QminError as err:
            # the reference's L-BFGS takes fixed steps (no line search, no
            # curvature test): a run can blow up, which ends it with a
            # non-finite force norm
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            out[tag] = {"time_s": dt, "diverged": True, "error": str(err), "iterations": err.iterations,
                        "site_steps_per_s": N * err.iterations / dt if err.iterations else None,
                        "params": "reference defaults (L-BFGS m 5 eta 1e-4)"}
            lat.close()
            continue
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        e, _ = lat.energy()
        out[tag] = {"time_s": dt, "iterations": r["iterations"], "forceMax": r["forceMax"],
                    "converged": r["forceMax"] < 1e-6, "E_per_site": e,
                    "site_steps_per_s": N * r["iterations"] / dt,
                    "params": "reference defaults (Adam b1 .9 b2 .99 eps 1e-8 dt 1e-4; L-BFGS m 5 eta 1e-4)"}
        lat.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-sample-iters", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the c1 and c3 runs")
    ap.add_argument("--lattice", type=int, default=200, help="cube side (profiling of smaller cases)")
    ap.add_argument("--forms", default="both", choices=["both", "fp64", "fp32"])
    ap.add_argument("--workload", default="c2", choices=["c2", "c2-converge", "c3", "c5", "warmnet", "kernels"],
                    help="c3: the batched uneven solves alone; c5: the 400^3 multi-sphere E-field case; "
                         "warmnet: the warm-start net's forward pass; kernels: one small call of every kernel family "
                         "(for profilers)")
    ap.add_argument("--families", default="fp64,fp32,onec,batch,batchmc,net",
                    help="kernels workload: comma-separated families (fp64, fp32, onec, batch, batchmc, net)")
    ap.add_argument("--warmnet-weights", default=None, help="warm-start weights file (default: the committed c4 weights)")
    ap.add_argument("--c3-solves", type=int, default=512, help="c3: number of solves (profiling of smaller cases)")
    ap.add_argument("--c3-max-iterations", type=int, default=30000)
    ap.add_argument("--c5-max-iterations", type=int, default=20000)
    ap.add_argument("--c5-fire-only", action="store_true", help="c5: FIRE and the warm start only (no Adam, L-BFGS)")
    ap.add_argument("--c4-test", type=int, default=64, help="c4 test solves for the warm-start protocol (0: skip)")
    # a fixed FIRE strategy instead of the autotuner's choice (for profiling runs, where the
    # profiler's serialised launches would bias the autotuner's timings)
    ap.add_argument("--fire-kernel-fp64", default="auto", choices=["auto", "separate", "fused", "split"])
    ap.add_argument("--fire-kernel-fp32", default="auto", choices=["auto", "separate", "fused", "tiled", "split"])
    ap.add_argument("--fire-variant-fp64", type=int, default=-1, help="variant index of the pinned FP64 strategy")
    ap.add_argument("--fire-variant-fp32", type=int, default=-1, help="variant index of the pinned FP32 strategy")
    args = ap.parse_args()
    if args.warmnet_weights:
        global WARMNET_WEIGHTS
        WARMNET_WEIGHTS = os.path.abspath(args.warmnet_weights)
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.workload == "c5":
        if rank == 0:
            print(json.dumps(run_c5(args)))
        return 0
    if args.lattice != 200:
        scale_workload(args.lattice)
    if args.workload == "warmnet":
        if rank == 0:
            print(json.dumps(run_warmnet(args)))
        return 0
    if args.workload == "kernels":
        if rank == 0:
            print(json.dumps(run_kernels(args)))
        return 0
    if args.workload == "c2-converge":
        # time to forceMax < 1e-6 on the 200^3 workload only: plain FP64, plain
        # FP32 and the learned warm start under the protocol
        if rank == 0:
            import __graft_entry__ as ge
            q = ge.load_package()
            consts, g = build_workload_host(q)
            t64 = time_to_converge(q, consts, g, q.FP64)
            t32 = time_to_converge(q, consts, g, q.FP32)
            out = {"workload": "200^3 c2, FIRE to forceMax < 1e-6", "fp64": t64, "fp32_form": t32}
            if os.path.exists(WARMNET_WEIGHTS):
                out["warm_start_fp32"] = warm_start_c2(q, consts, g, t64, t32)
            print(json.dumps(out))
        return 0
    if args.workload == "c3":
        if rank == 0:
            import __graft_entry__ as ge
            print(json.dumps(run_c3(ge.load_package(), args.c3_solves, args.c3_max_iterations)))
        return 0

    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args)))
        return 0

    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        torch.distributed.init_process_group("nccl")
    out = run_ours(args, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline and args.forms == "both":
            out["cpu_baseline"], r_or, q_or = cpu_baseline(args.cpu_sample_iters)
            import __graft_entry__ as ge
            out["cpu_baseline"].update(c2_parity(ge.load_package(), args.cpu_sample_iters, r_or, q_or))
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
