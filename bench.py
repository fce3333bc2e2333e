#!/usr/bin/env python
"""Benchmark: rays/s of batched tracing on one GB300 (256 sun positions of the 10,000-heliostat field).

Headline workload (default, `--workload batched`): the 10,000-heliostat radial-stagger field
(10 x 10 m flat mirrors, cylindrical receiver r = 8 m, h = 20 m at 200 m; pillbox sun 4.65 mrad;
slope error 1.5 mrad) at 256 sun positions (elevation U(10, 80) deg, azimuth U(-120, 120) deg,
seed 2), every heliostat re-aimed per instance, ray counts log-uniform in [2^20, 2^25] (seed 3):
2,343,992,611 rays, float32, synthetic (the reference ships no benchmark scenes).

One step = one csp_batch run of all 256 instances: per-instance BVH refit and sun planes, one
persistent trace launch, receiver flux maps accumulated in the shading stage.

  value      rays/s with the instances' records resident in HBM: device time of K runs (refit, sun
             planes and trace, CUDA events inside the run's graph); the instances' scenes
             (~0.5 GB) exceed L2, so no flush is needed between steps.
  e2e        rays/s through the C ABI from host memory: K pipelined runs (csp_batch_run_async /
             csp_batch_wait) from the host pose arrays (element builds, staging, H2D upload) to the
             flux maps in host memory, wall clock.
  roofline   issue slots (nothing per ray leaves the SM: the batch kernel is bound by instruction
             issue and latency, not HBM): warp instructions per ray from ncu x rays / device time
             against SMs x 4 schedulers x the SM clock.
  cpu_baseline  the oracle port of the reference algorithm on all host cores, on ray samples of
             the batched workload's instances (brute-force closest hit over 10,001 elements).
  plain_loop the same instances through the drop-in handle one scene at a time (new poses,
             csp_update, csp_run, csp_flux_map): the plain per-scene launch loop the batched and
             served modes are measured against.

The default line also carries the plain trace workloads and the served workload as sub-objects:
`single_parabolic` (one parabolic heliostat, 16M rays, the dense-record HBM roofline),
`large_field` (the field in one plain launch of 268M rays) and `served` (Poisson requests over
fields of 3 / 1,000 / 10,000 heliostats through csp_server, p50 / p99 latency).  `--workload
single_parabolic|three_heliostats|large_field|served` prints one of those as the whole line;
`--no-systems` leaves the sub-objects out.

--impl reference times the reference algorithm's CPU implementation (the oracle port: the
reference's own programs cannot run the slope error and re-aiming of this workload) on all host
cores, on the same workload and metric.

Multi-GPU: replicas only (each rank traces its own copy of the workload; no exchange), launched by
torchrun; value = all rays / max-over-ranks time.
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

METRIC = "rays/s on 1 GB300 (batched/served vs plain trace) at flux L2<=1%; p50/p99 latency"
BYTES_PER_RAY = 80  # 5 float4 hit records per ray, fully rewritten by every plain trace
# dram__bytes_read.sum + dram__bytes_write.sum of the single parabolic workload's trace_kernel per
# launch of 16,777,216 rays: 4 x (8,776,704 + 291,551,232) bytes, scaled by the rays from
# `ncu --set full -k regex:^trace_kernel -s 2 -c 1` of `python bench.py --workload single_parabolic
# --rays 4194304 --steps 2 --warmup 2 --no-cpu-baseline --no-accuracy --e2e-steps 0` (the record
# stream grows with the rays; at that size ~35 MB of the last records are still in L2 when the
# kernel ends)
NCU_TRAFFIC_PER_LAUNCH = 4 * (8776704 + 291551232)
# The same for the field kernel (trace_kernel<grid>) of the 10,000-heliostat field per launch of
# 268,435,456 rays: 64 x (15,834,112 + 297,401,344) bytes from `ncu --set full -k regex:^trace_kernel
# -s 2 -c 1` of `python bench.py --workload large_field --rays 4194304 --steps 2 --warmup 2
# --no-cpu-baseline --no-accuracy --e2e-steps 0`, scaled by the rays
NCU_TRAFFIC_PER_LAUNCH_FIELD = 64 * (15834112 + 297401344)
# Batch kernel (field grid) on the batched workload: warp instructions and DRAM bytes per traced ray,
# from `ncu --set full -k regex:^batch_kernel -s 2 -c 1` of `python bench.py --workload batched
# --instances 8 --tuning 256,4,256 --steps 1 --warmup 3 --no-systems --no-cpu-baseline
# --plain-instances 1` (one launch over 42,028,566 rays): smsp__inst_executed.sum = 3,229,355,334
# and dram__bytes_read.sum + dram__bytes_write.sum = 52,126,464 + 1,675,776 bytes, per ray.
BATCH_WARP_INST_PER_RAY = 3229355334 / 42028566
BATCH_DRAM_BYTES_PER_RAY = (52126464 + 1675776) / 42028566
ISSUE_PER_SM_PER_CYCLE = 4  # one warp instruction per cycle per scheduler, 4 schedulers per SM


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=None, help="timed steps (default: 10 batched, 400 plain)")
    p.add_argument("--warmup", type=int, default=None, help="warm-up steps (default: 3 batched, 10 plain)")
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--rays", type=int, default=None, help="ray count (default: the workload's)")
    p.add_argument("--workload", choices=["batched", "single_parabolic", "three_heliostats", "large_field", "served"],
                   default="batched", help="batched is the benchmark line; the others are reported inside it")
    p.add_argument("--instances", type=int, default=256, help="batched workload: number of instances")
    p.add_argument("--heliostats", type=int, default=10000, help="batched / large_field: field size")
    p.add_argument("--e2e-steps", type=int, default=10)
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-accuracy", action="store_true")
    p.add_argument("--no-systems", action="store_true",
                   help="batched line without the plain and served sub-objects")
    p.add_argument("--tuning", type=str, default="", help="batched workload: block,ctas_per_sm,chunk (default: autotune)")
    p.add_argument("--requests", type=int, default=300, help="served workload: number of requests")
    p.add_argument("--rate", type=float, default=200.0, help="served workload: Poisson arrival rate (1/s)")
    p.add_argument("--plain-instances", type=int, default=0,
                   help="batched workload: instances timed in the plain loop (0 = all)")
    a = p.parse_args()
    plain = a.workload in ("single_parabolic", "three_heliostats", "large_field")
    if a.steps is None:
        a.steps = 400 if plain and a.workload != "large_field" else 10
    if a.warmup is None:
        a.warmup = 10 if plain else 3
    return a


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    """(HBM GB/s, source, SM max MHz) from the measured peaks, else the fallback figures."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured", float(d.get("sm_max_mhz", 2070.0))
    except Exception:
        return 6800.0, "fallback", 2070.0


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "100"], stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(seconds: float, pg, device: str) -> float:
    """Replica timing: the largest of every rank's seconds (the job ends with its slowest replica);
    the value itself when there is no process group."""
    if pg is None:
        return seconds
    import torch
    t = torch.tensor([seconds], device=device, dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())




def _cpu_trace_for(seconds: float, jobs, sample: int):
    """Oracle port of the reference algorithm on all host cores: `sample`-ray windows of the jobs
    (elements, sun, shape, param, rays) round robin for about `seconds`.  Returns (rays, s, cores)."""
    from oracle import oracle
    oracle.build(with_ref=False)
    o = oracle.Oracle("f32")
    cores = os.cpu_count() or 1
    el, sun, shape, param, n = jobs[0]
    o.trace(el, sun, shape, param, count=max(1, sample // 8), nthreads=cores, with_ids=False)
    done, k, t0 = 0, 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        el, sun, shape, param, n = jobs[k % len(jobs)]
        first = ((k // len(jobs)) * sample) % max(1, n - sample + 1)
        o.trace(el, sun, shape, param, first_ray=first, count=sample, nthreads=cores, with_ids=False)
        done += sample
        k += 1
    return done, time.perf_counter() - t0, cores


def cpu_baseline(seconds: float, jobs, sample: int, what: str):
    done, dt, cores = _cpu_trace_for(seconds, jobs, sample)
    return {"value": done / dt, "unit": "rays/s", "cores": cores, "kind": "port",
            "sample": f"{done} rays ({done // sample} windows of {sample}) of the {what} workload, {dt:.1f} s, "
                      f"oracle port of the reference algorithm, OpenMP over {cores} threads"}


def make_scene(workload, rays):
    from optixsoltracedemos_gb300 import scenes
    if workload == "three_heliostats":
        sc = scenes.three_heliostats()
    elif workload == "large_field":
        sc = scenes.large_field()
    else:
        sc = scenes.single_parabolic()
    if rays:
        sc.num_rays = rays
    return sc


def config(sc):
    rays = sc.num_rays
    base = {"rays": rays, "elements": int(len(sc.elements)), "hit_buffer_bytes": rays * BYTES_PER_RAY,
            "l2_policy": f"hit buffer ({rays * BYTES_PER_RAY / 1e9:.2f} GB) larger than L2; no flush needed between steps",
            "parallelism": "replicas"}
    if sc.name == "single_parabolic":
        base.update({"workload": "single_parabolic_heliostat_cylinder_receiver", "sun": "gaussian 2.5 mrad",
                     "slope_error_rad": 1.5e-3, "focal_length_m": 100.0})
    elif sc.name == "three_heliostats":
        base.update({"workload": "three_flat_heliostats_flat_receiver", "sun": "pillbox 4.65 mrad",
                     "slope_error_rad": 1e-3, "reflectivity": 0.9})
    else:
        base.update({"workload": "large_field_10000_flat_heliostats_cylinder_receiver", "sun": "pillbox 4.65 mrad",
                     "slope_error_rad": 1.5e-3})
    return base


def batched_workload(n_instances, n_heliostats):
    """The large field at per-instance sun positions with re-aimed heliostats and log-uniform ray
    counts: (base elements, poses per instance, suns, ray counts)."""
    from optixsoltracedemos_gb300 import scenes
    base = scenes.large_field(n_heliostats=n_heliostats, num_rays=1).elements
    suns, counts = scenes.batched_instances(n_instances=n_instances, n_heliostats=n_heliostats)
    poses = [scenes.reaim(base, s) for s in suns]
    return base, poses, suns, counts


def batched_config(n_inst, n_heliostats, counts, extra=None):
    cfg = {"workload": f"batched_{n_inst}_instances_large_field_{n_heliostats}_heliostats",
           "instances": n_inst, "rays_total": int(counts.sum()), "rays_min": int(counts.min()),
           "rays_max": int(counts.max()), "flux_grid": [100, 100], "sun": "pillbox 4.65 mrad, elevation U(10,80) "
           "azimuth U(-120,120), heliostats re-aimed per instance", "slope_error_rad": 1.5e-3,
           "l2_policy": "per-instance scene data (element records, field grids, sun-ray grids: ~2.5 GB for "
                        "256 instances) exceed L2; no per-ray buffers",
           "parallelism": "replicas"}
    cfg.update(extra or {})
    return cfg


def served_workload(n_requests, rate):
    """Requests over resident scenes of 3, 1,000 and 10,000 heliostats, flat and parabolic (focal
    length 100 m): Poisson arrivals (seed 4), per-request sun (elevation U(10, 80), azimuth
    U(-120, 120) deg) with the heliostats re-aimed, ray counts log-uniform in [2^20, 2^26] (seed 5).
    Returns (scene element arrays, requests (scene, poses, sun, rays, arrival s))."""
    import math
    import numpy as np
    from optixsoltracedemos_gb300 import scenes
    th = scenes.three_heliostats().elements
    thp = th.copy()
    thp["surface"][:3] = scenes.SURFACE_PARABOLIC
    thp["curv_x"][:3] = thp["curv_y"][:3] = 1.0 / 200.0
    scene_list = [th, thp]
    for n in (1000, 10000):
        for par in (False, True):
            scene_list.append(scenes.large_field(n_heliostats=n, parabolic=par, num_rays=1).elements)
    ra = np.random.default_rng(4)
    arrivals = np.cumsum(ra.exponential(1.0 / rate, n_requests))
    rs = np.random.default_rng(5)
    reqs = []
    for k in range(n_requests):
        sid = int(rs.integers(0, len(scene_list)))
        sun = scenes.sun_vector(rs.uniform(10.0, 80.0), rs.uniform(-120.0, 120.0))
        rays = int(math.exp(rs.uniform(20 * math.log(2), 26 * math.log(2))))
        reqs.append((sid, scenes.reaim(scene_list[sid], sun), sun, rays, float(arrivals[k])))
    return scene_list, reqs


def workload_jobs(args):
    """CPU jobs (elements, sun, shape, param, rays), config and window size of the workload."""
    from optixsoltracedemos_gb300 import scenes
    if args.workload == "batched":
        _, poses, suns, counts = batched_workload(args.instances, args.heliostats)
        jobs = [(poses[i], suns[i], scenes.SUN_PILLBOX, 4.65e-3, int(counts[i])) for i in range(len(suns))]
        return jobs, batched_config(len(suns), args.heliostats, counts), 1 << 14
    if args.workload == "served":
        _, reqs = served_workload(args.requests, args.rate)
        jobs = [(p, sun, scenes.SUN_PILLBOX, 4.65e-3, rays) for (_, p, sun, rays, _) in reqs]
        cfg = {"workload": "served_requests_fields_3_1000_10000_flat_parabolic", "requests": len(reqs),
               "rays_total": int(sum(j[4] for j in jobs))}
        return jobs, cfg, 1 << 14
    sc = make_scene(args.workload, args.rays)
    jobs = [(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, sc.num_rays)]
    sample = min(1 << 20, sc.num_rays) if args.workload != "large_field" else 1 << 14
    return jobs, config(sc), sample


def run_reference(args):
    """The reference algorithm's CPU implementation (oracle port) on all host cores, on the same
    workload: each step traces one window of rays of the next instance / request / scene."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle
    oracle.build(with_ref=False)
    o = oracle.Oracle("f32")
    cores = os.cpu_count() or 1
    jobs, cfg, sample = workload_jobs(args)

    def step(k):
        el, sun, shape, param, n = jobs[k % len(jobs)]
        first = ((k // len(jobs)) * sample) % max(1, n - sample + 1)
        o.trace(el, sun, shape, param, first_ray=first, count=sample, nthreads=cores, with_ids=False)

    for w in range(args.warmup):
        step(w)
    t0 = time.perf_counter()
    for k in range(args.steps):
        step(k)
    dt = time.perf_counter() - t0
    v = args.steps * sample / dt
    what = (f"each step traces {sample} rays of the next instance / request (brute-force closest hit over its "
            f"elements)" if args.workload in ("batched", "served") else f"each step traces {sample} rays of the scene")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "rays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": cfg,
            "cpu_baseline": {"value": v, "unit": "rays/s", "cores": cores, "kind": "port",
                             "sample": f"{what} (oracle port of the reference algorithm, OpenMP over {cores} threads)"},
            "e2e": {"value": v, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def measure_write_output(sc, local, n):
    """The reference's write_output end to end (lib/soltrace_system.cpp:208-264): trace, records to
    the host, the CSV file written; dense records (csp_run_to_host + csp_write_hits_csv) against
    compact ones (csp_run_to_host_compact + csp_write_compact_csv), the file the same."""
    import numpy as np
    from optixsoltracedemos_gb300 import native
    tr = native.tracer_for(sc, device=local, record_ids=False, num_rays=n)
    out = {"rays": n, "unit": "rays/s"}
    with tempfile.TemporaryDirectory() as d:
        dense = np.empty((n, 5, 4), np.float32)
        pts, cnt, rec = np.empty((n, 3), np.float32), np.empty(n, np.uint8), np.empty((4 * n, 4), np.float32)
        best_d = best_c = 1e30
        for _ in range(2):
            t0 = time.perf_counter()
            tr.run_to_host(dense.reshape(-1))
            native.write_hits_csv(dense, os.path.join(d, "dense.csv"))
            best_d = min(best_d, time.perf_counter() - t0)
            t0 = time.perf_counter()
            p, c, r = tr.run_to_host_compact(pts, cnt, rec)
            native.write_compact_csv(p, c, r, os.path.join(d, "compact.csv"))
            best_c = min(best_c, time.perf_counter() - t0)
        size = os.path.getsize(os.path.join(d, "dense.csv"))
        same = open(os.path.join(d, "dense.csv"), "rb").read() == open(os.path.join(d, "compact.csv"), "rb").read()
    tr.close()
    out.update({"dense_rays_per_s": n / best_d, "compact_rays_per_s": n / best_c, "csv_bytes": size,
                "csv_identical": same, "host_threads": os.cpu_count()})
    return out


def measure_plain(args, sc, local, world, pg, steps, warmup, e2e_steps, accuracy, cpu_seconds, write_output_rays=0):
    """Plain trace of one scene: K launches with the scene resident (CUDA events on the launching
    stream), the end-to-end rate through the C ABI with host buffers, the HBM roofline of the dense
    record stream, and the flux-map L2 against the FP64 oracle."""
    import torch
    from optixsoltracedemos_gb300 import native
    from optixsoltracedemos_gb300.flux import flux_map_from_hits, flux_l2

    rank = int(os.environ.get("RANK", "0"))
    N = sc.num_rays
    tr = native.tracer_for(sc, device=local, record_ids=False)
    stream = torch.cuda.Stream(device=local)
    sp = stream.cuda_stream
    for w in range(warmup):
        tr.set_seed(w)
        tr.trace_async(sp)
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    clk = ClockSampler(local)
    clk.start()
    time.sleep(0.3)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for k in range(steps):
        tr.set_seed(1000 + k, rank)  # each replica traces its own rays (Philox instance = rank)
        starts[k].record(stream)
        tr.trace_async(sp)
        ends[k].record(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    total_s = max_over_ranks(e0.elapsed_time(e1) * 1e-3, pg, f"cuda:{local}")
    launch_s = statistics.mean(s.elapsed_time(e) for s, e in zip(starts, ends)) * 1e-3
    peak, peak_kind, _ = peaks()
    achieved = BYTES_PER_RAY * N / launch_s / 1e9
    line = {
        "metric": METRIC, "value": world * N * steps / total_s, "unit": "rays/s", "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": total_s / steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config(sc),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": (NCU_TRAFFIC_PER_LAUNCH if (N == 1 << 24 and sc.name == "single_parabolic") else
                                 NCU_TRAFFIC_PER_LAUNCH_FIELD if (N == 1 << 28 and sc.name == "large_field") else None),
                     "traffic_source": ("ncu dram bytes of a 4,194,304-ray launch x 4" if (
                         N == 1 << 24 and sc.name == "single_parabolic") else "ncu dram bytes of a 4,194,304-ray launch x 64"
                         if (N == 1 << 28 and sc.name == "large_field") else None),
                     "peak_source": peak_kind, "algorithmic_bytes_per_launch": BYTES_PER_RAY * N,
                     "launch_ms": launch_s * 1e3},
        "gpu_launches": steps, "clocks": clocks,
    }
    host = None
    if e2e_steps > 0:
        # end to end through the C ABI with host buffers: element list up, every record down
        host = torch.empty(N * 5 * 4, dtype=torch.float32, pin_memory=True)
        elements = sc.elements.copy()
        for _ in range(2):
            tr.set_elements(elements)
            tr.update()
            tr.run_to_host_ptr(host.data_ptr())
        if pg:
            pg.barrier()
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            tr.set_seed(5000 + k, rank)
            tr.set_elements(elements)
            tr.update()
            tr.run_to_host_ptr(host.data_ptr())
        e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, pg, f"cuda:{local}")
        line["e2e"] = {"value": world * N / e2e_s, "unit": "rays/s", "h2d_bytes_per_step": int(elements.nbytes + 3 * 8),
                       "d2h_bytes_per_step": int(N * BYTES_PER_RAY)}
        # the same end to end with the compact record transfer (csp_run_to_host_compact): per ray its
        # sun-plane point and record count, then only the records that exist
        pts = torch.empty(N * 3, dtype=torch.float32, pin_memory=True)
        cnt = torch.empty(N, dtype=torch.uint8, pin_memory=True)
        cap = 4 * N
        rec = torch.empty(cap * 4, dtype=torch.float32, pin_memory=True)
        nrec = tr.run_to_host_compact_ptr(pts.data_ptr(), cnt.data_ptr(), rec.data_ptr(), cap)
        if pg:
            pg.barrier()
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            tr.set_seed(5000 + k, rank)
            tr.set_elements(elements)
            tr.update()
            nrec = tr.run_to_host_compact_ptr(pts.data_ptr(), cnt.data_ptr(), rec.data_ptr(), cap)
        ec_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, pg, f"cuda:{local}")
        line["e2e_compact"] = {"value": world * N / ec_s, "unit": "rays/s",
                               "h2d_bytes_per_step": int(elements.nbytes + 3 * 8),
                               "d2h_bytes_per_step": int(13 * N + 16 * nrec),
                               "path": "csp_run_to_host_compact: sun-plane points, record counts, existing records"}
        del pts, cnt, rec
    if rank == 0 and world == 1 and accuracy and host is not None:
        try:
            from oracle import oracle
            oracle.build(with_ref=False)
            tr.set_seed(0)
            hits = host.numpy().reshape(N, 5, 4)
            tr.run_to_host(hits.reshape(-1))
            o64 = oracle.Oracle("f64")
            oh, _ = o64.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, count=N, with_ids=False)
            line["flux_l2_vs_fp64"] = flux_l2(flux_map_from_hits(hits, sc.elements[-1], N),
                                              flux_map_from_hits(oh, sc.elements[-1], N))
            del oh
        except Exception as exc:  # accuracy is reported, not required for the timing line
            line["flux_l2_vs_fp64"] = f"unavailable: {exc}"
    if rank == 0 and world == 1 and write_output_rays > 0:
        line["write_output"] = measure_write_output(sc, local, min(N, write_output_rays))
    if rank == 0 and world == 1 and cpu_seconds > 0:
        sample = min(1 << 20, N) if len(sc.elements) < 64 else 1 << 12
        line["cpu_baseline"] = cpu_baseline(cpu_seconds, [(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, N)],
                                            sample, sc.name)
    tr.close()
    return line


def measure_batched(args, local, world, pg=None):
    """Batched workload through csp_batch: K synchronous runs (device time of refit, sun planes and
    trace per run, CUDA events inside the run's graph), K pipelined runs from host poses to host
    flux maps (run_async / wait: the host builds of one run overlap the device work of the
    previous one), and the plain per-scene loop through the drop-in handle (per instance: new poses
    and sun, csp_update, csp_run, csp_flux_map) on the same instances, flux maps compared."""
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    from optixsoltracedemos_gb300 import native, scenes

    base, poses, suns, counts = batched_workload(args.instances, args.heliostats)
    total = int(counts.sum())
    steps, warmup = args.steps, max(1, args.warmup)
    b = native.Batch(local)
    sid = b.add_scene(base)
    rank = int(os.environ.get("RANK", "0"))
    for i in range(len(suns)):
        b.add_instance(sid, suns[i], scenes.SUN_PILLBOX, 4.65e-3, int(counts[i]), seed=rank, instance=i,
                       poses=poses[i])
    if args.tuning:
        b.set_tuning(*[int(x) for x in args.tuning.split(",")])
    t0 = time.perf_counter()
    b.run()  # autotune (first run of this scene class) + graph capture
    first_s = time.perf_counter() - t0
    for _ in range(warmup - 1):
        b.run()
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    clk = ClockSampler(local)
    clk.start()
    time.sleep(0.2)
    wall, dev = [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        b.run()
        wall.append(time.perf_counter() - t0)
        dev.append(b.timing()[1])
    torch.cuda.synchronize()
    batch_counts = [b.counts(i).copy() for i in range(len(suns))]
    # pipelined from host memory: K runs, first submission to last completion
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    b.run_async()
    for _ in range(steps - 1):
        b.run_async()
        b.wait()
    b.wait()
    piped_s = time.perf_counter() - t0
    clocks = clk.stop()
    h2d, d2h = b.transfer()
    piped_mismatch = sum(int(not np.array_equal(b.counts(i), batch_counts[i])) for i in range(len(suns)))
    dev_s = max_over_ranks(sum(dev), pg, f"cuda:{local}")
    piped_s = max_over_ranks(piped_s, pg, f"cuda:{local}")

    # plain per-scene loop through the drop-in handle
    tr = native.Tracer(local, int(counts.max()))
    tr.set_elements(poses[0])
    tr.set_sun_vector(suns[0])
    tr.set_sun_shape(scenes.SUN_PILLBOX, 4.65e-3)
    tr.initialize()
    n_plain = len(suns) if args.plain_instances <= 0 else min(len(suns), args.plain_instances)
    mismatches = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(n_plain):
        tr.set_elements(poses[i])
        tr.set_sun_vector(suns[i])
        tr.set_num_rays(int(counts[i]))
        tr.set_seed(rank, i)
        tr.update()
        tr.run()
        c, _ = tr.flux_map()
        mismatches += int(not np.array_equal(c, batch_counts[i]))
    plain_s = time.perf_counter() - t0
    plain_rays = int(counts[:n_plain].sum())
    tr.close()
    tg, tl = b.tuning(native.GROUP_GRID), b.tuning(native.GROUP_BVH)
    b.close()

    value = world * total * steps / dev_s
    _, _, sm_mhz = peaks()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    issue_peak = sms * ISSUE_PER_SM_PER_CYCLE * sm_mhz * 1e6
    per_gpu = value / world
    roof = {"bound": "issue", "unit": "warp-inst/s", "peak": issue_peak,
            "peak_source": f"{sms} SMs x {ISSUE_PER_SM_PER_CYCLE} schedulers x {sm_mhz:.0f} MHz",
            "launch_ms": statistics.mean(dev) * 1e3, "rays_per_launch": total}
    if BATCH_WARP_INST_PER_RAY is not None:
        roof.update({"achieved": BATCH_WARP_INST_PER_RAY * per_gpu, "frac": BATCH_WARP_INST_PER_RAY * per_gpu / issue_peak,
                     "warp_inst_per_ray": BATCH_WARP_INST_PER_RAY})
    else:
        roof.update({"achieved": None, "frac": None})
    if BATCH_DRAM_BYTES_PER_RAY is not None:
        hbm, _, _ = peaks()
        roof.update({"traffic": BATCH_DRAM_BYTES_PER_RAY * total,
                     "hbm_frac": BATCH_DRAM_BYTES_PER_RAY * per_gpu / 1e9 / hbm})
    else:
        roof["traffic"] = None
    line = {
        "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": dev_s / steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": batched_config(len(suns), args.heliostats, counts, {"tuning_grid": tg, "tuning_bvh": tl}),
        "roofline": roof,
        "e2e": {"value": world * total * steps / piped_s, "unit": "rays/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "path": "csp_batch_run_async / csp_batch_wait from host pose arrays to host flux maps, pipelined"},
        # per run: refit, sun planes, the sun-ray grids' size / count / scan / fill, the batch kernel
        "gpu_launches": 7 * steps,
        "clocks": clocks,
        "batched_wall_rays_per_s": world * total / max_over_ranks(statistics.median(wall), pg, f"cuda:{local}"),
        "pipelined_flux_counts_mismatching": piped_mismatch,
        "first_run_s": first_s,
        "plain_loop": {"rays_per_s": plain_rays / plain_s, "instances": n_plain, "seconds": plain_s,
                       "flux_counts_mismatching_batched": mismatches,
                       "path": "drop-in handle per instance: csp_set_elements, csp_update, csp_run, csp_flux_map"},
        "speedup_vs_plain_loop": (total * steps / piped_s) / (plain_rays / plain_s),
        "speedup_vs_plain_loop_device": (total * steps / sum(dev)) / (plain_rays / plain_s),
    }
    return line


def measure_served(args, local, world):
    """Serving workload through csp_server (continuous batching) against the plain per-scene loop
    (one drop-in handle per scene: update, run, device flux map per request, in arrival order), at
    saturation (all requests queued at once) and with real-time Poisson arrivals."""
    import threading
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    from optixsoltracedemos_gb300 import native, scenes

    scene_list, reqs = served_workload(args.requests, args.rate)
    total = sum(r[3] for r in reqs)

    def serve(realtime: bool):
        srv = native.Server(local, memory_budget=16 << 30, max_active=64)
        sids = [srv.add_scene(e) for e in scene_list]
        # warm up every scene once (first-launch costs)
        for sid in sids:
            srv.wait(srv.submit(sid, reqs[0][2], scenes.SUN_PILLBOX, 4.65e-3, 1 << 16))
        ids = [None] * len(reqs)
        lat = [None] * len(reqs)
        t0 = time.perf_counter()

        def submitter():
            for k, (sid, poses, sun, rays, at) in enumerate(reqs):
                if realtime:
                    d = t0 + at - time.perf_counter()
                    if d > 0:
                        time.sleep(d)
                ids[k] = srv.submit(sids[sid], sun, scenes.SUN_PILLBOX, 4.65e-3, rays, seed=k, instance=k,
                                    poses=poses)
        th = threading.Thread(target=submitter)
        th.start()
        counts = []
        for k in range(len(reqs)):
            while ids[k] is None:
                time.sleep(1e-4)
            c, st, l = srv.wait(ids[k])
            counts.append(c)
            lat[k] = l[0]
        t1 = time.perf_counter()
        th.join()
        srv.close()
        return {"seconds": t1 - t0, "rays_per_s": total / (t1 - t0), "p50_s": float(np.percentile(lat, 50)),
                "p99_s": float(np.percentile(lat, 99))}, counts

    def plain(realtime: bool, ref_counts=None):
        tracers = []
        for e in scene_list:
            t = native.Tracer(local, 1 << 26)  # hit buffer sized for the largest request up front
            t.set_elements(e)
            t.set_sun_vector(reqs[0][2])
            t.set_sun_shape(scenes.SUN_PILLBOX, 4.65e-3)
            t.initialize()
            t.run()
            tracers.append(t)
        lat, mism = [], 0
        t0 = time.perf_counter()
        for k, (sid, poses, sun, rays, at) in enumerate(reqs):
            if realtime:
                d = t0 + at - time.perf_counter()
                if d > 0:
                    time.sleep(d)
            t = tracers[sid]
            t.set_elements(poses)
            t.set_sun_vector(sun)
            t.set_num_rays(rays)
            t.set_seed(k, k)
            t.update()
            t.run()
            c, _ = t.flux_map()
            if ref_counts is not None:
                mism += int(not np.array_equal(c, ref_counts[k]))
            lat.append(time.perf_counter() - (t0 + at if realtime else t0))
        t1 = time.perf_counter()
        for t in tracers:
            t.close()
        return {"seconds": t1 - t0, "rays_per_s": total / (t1 - t0), "p50_s": float(np.percentile(lat, 50)),
                "p99_s": float(np.percentile(lat, 99)), "flux_counts_mismatching_served": mism}

    clk = ClockSampler(local)
    clk.start()
    time.sleep(0.2)
    sat, counts = serve(False)
    rt, _ = serve(True)
    clocks = clk.stop()
    psat = plain(False, counts)
    prt = plain(True)
    line = {
        "metric": METRIC, "value": sat["rays_per_s"], "unit": "rays/s", "n_gpus": world, "steps": len(reqs),
        "warmup": len(scene_list), "ms_per_step": sat["seconds"] / len(reqs) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "served_requests_fields_3_1000_10000_flat_parabolic", "requests": len(reqs),
                   "rays_total": total, "arrival_rate_per_s": args.rate, "rays_per_request": "log-uniform [2^20, 2^26]",
                   "sun": "pillbox 4.65 mrad, per-request elevation U(10,80) azimuth U(-120,120), heliostats re-aimed",
                   "flux_grid": [100, 100], "max_active": 64,
                   "l2_policy": "per-request scenes and flux maps; no per-ray buffers"},
        "served_saturation": sat, "served_poisson": rt,
        "plain_loop_saturation": psat, "plain_loop_poisson": prt,
        "speedup_vs_plain_loop": sat["rays_per_s"] / psat["rays_per_s"],
        "e2e": {"value": sat["rays_per_s"], "unit": "rays/s",
                "h2d_bytes_per_step": int(sum(r[1].nbytes for r in reqs) / len(reqs)),
                "d2h_bytes_per_step": 100 * 100 * 4},
        "gpu_launches": None,
        "clocks": clocks,
    }
    return line


def _plain_summary(line):
    keep = ("value", "ms_per_step", "roofline", "e2e", "e2e_compact", "write_output", "flux_l2_vs_fp64", "cpu_baseline",
            "clocks")
    out = {"workload": line["config"]["workload"], "rays": line["config"]["rays"], "unit": "rays/s"}
    out.update({k: line[k] for k in keep if k in line})
    out["rays_per_s"] = out.pop("value")
    return out


def _served_summary(v):
    return {"workload": v["config"]["workload"], "requests": v["config"]["requests"], "rays": v["config"]["rays_total"],
            "saturation_rays_per_s": v["served_saturation"]["rays_per_s"],
            "plain_loop_saturation_rays_per_s": v["plain_loop_saturation"]["rays_per_s"],
            "speedup_vs_plain_loop": v["speedup_vs_plain_loop"], "poisson_rate_per_s": v["config"]["arrival_rate_per_s"],
            "poisson_p50_s": v["served_poisson"]["p50_s"], "poisson_p99_s": v["served_poisson"]["p99_s"],
            "plain_loop_poisson_p50_s": v["plain_loop_poisson"]["p50_s"],
            "plain_loop_poisson_p99_s": v["plain_loop_poisson"]["p99_s"],
            "flux_counts_mismatching_plain": v["plain_loop_saturation"]["flux_counts_mismatching_served"]}


def run_ours(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist

    from optixsoltracedemos_gb300 import build as nbuild
    if rank == 0:
        nbuild.build()
    if pg:
        pg.barrier()
    from optixsoltracedemos_gb300 import native
    native.load()

    solo = rank == 0 and world == 1
    if args.workload == "batched":
        line = measure_batched(args, local, world, pg)
        if solo and not args.no_cpu_baseline:
            jobs, _, sample = workload_jobs(args)
            line["cpu_baseline"] = cpu_baseline(args.cpu_seconds, jobs, sample, line["config"]["workload"])
        if world == 1 and not args.no_systems:
            sub = argparse.Namespace(**vars(args))
            sc = make_scene("single_parabolic", None)
            line["single_parabolic"] = _plain_summary(measure_plain(
                sub, sc, local, world, pg, steps=200, warmup=10, e2e_steps=5, accuracy=not args.no_accuracy,
                cpu_seconds=0.0 if args.no_cpu_baseline else 3.0, write_output_rays=1 << 22))
            sc = make_scene("large_field", None)
            line["large_field"] = _plain_summary(measure_plain(
                sub, sc, local, world, pg, steps=5, warmup=3, e2e_steps=0, accuracy=False, cpu_seconds=0.0))
            line["served"] = _served_summary(measure_served(sub, local, world))
    elif args.workload == "served":
        line = measure_served(args, local, world)
    else:
        sc = make_scene(args.workload, args.rays)
        e2e_steps = args.e2e_steps if sc.num_rays <= (1 << 26) else 0
        line = measure_plain(args, sc, local, world, pg, args.steps, args.warmup, e2e_steps,
                             not args.no_accuracy and sc.num_rays <= (1 << 24),
                             0.0 if args.no_cpu_baseline else args.cpu_seconds,
                             write_output_rays=(1 << 22) if e2e_steps > 0 else 0)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
