#!/usr/bin/env python
"""Benchmark: rays/s of the plain trace on one GB300 (single parabolic heliostat workload).

Workload (default): 10 x 10 m paraboloid (focal length 100 m) at (0,100,0) aimed at a cylindrical
receiver r = 2 m, h = 4 m centred (0,0,100); Gaussian sun 2.5 mrad; slope error 1.5 mrad;
16,777,216 rays, float32, synthetic (the reference ships no benchmark scenes).

One step = one trace of all rays: generation, closest-hit search, shading, and the full rewrite of
the dense 16M x 5 float4 hit buffer (1.34 GB, larger than L2, so no flush is needed between steps).

  value      rays/s with the scene resident in HBM: K trace launches timed with CUDA events on the
             launching stream.
  e2e        rays/s through the public C ABI with host buffers: per step, upload of the element list
             (csp_set_elements + csp_update: H2D, refit, sun plane) and csp_run_to_host (trace +
             D2H of every hit record into page-locked memory), wall-clock timed.
  roofline   HBM: algorithmic bytes = 80 B per ray (the dense hit records) / per-launch time.
  cpu_baseline  the oracle port of the reference algorithm on all host cores, bounded sample.

The default line also carries `batched` (256 sun positions of the 10,000-heliostat field, one
csp_batch run, against the plain per-scene loop through the drop-in handle) and `served` (300
requests over fields of 3 / 1,000 / 10,000 heliostats through csp_server, at saturation and with
Poisson arrivals at 200/s: p50 / p99 latency, against the plain loop); `--workload batched|served`
prints those lines in full, `--no-systems` leaves them out.

--impl reference times the reference algorithm's CPU implementation (the oracle port: the
reference's own programs cannot run this workload's Gaussian sun and slope error) on all host
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
BYTES_PER_RAY = 80  # 5 float4 hit records per ray, fully rewritten by every trace
# dram__bytes_read.sum + dram__bytes_write.sum of one full-size trace_kernel launch of this workload
# (34,487,552 + 1,318,957,568 bytes), from the ncu capture summarised in
# profiles/trace_kernel_single_parabolic.md
NCU_TRAFFIC_PER_LAUNCH = 1371278592


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=400)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--rays", type=int, default=None, help="ray count (default: the workload's)")
    p.add_argument("--workload", choices=["single_parabolic", "three_heliostats", "large_field", "batched", "served"],
                   default="single_parabolic",
                   help="single_parabolic is the benchmark line; the others are for reporting only")
    p.add_argument("--instances", type=int, default=256, help="batched workload: number of instances")
    p.add_argument("--heliostats", type=int, default=10000, help="batched / large_field: field size")
    p.add_argument("--e2e-steps", type=int, default=10)
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-accuracy", action="store_true")
    p.add_argument("--no-systems", action="store_true",
                   help="default line without the batched and served summaries")
    p.add_argument("--tuning", type=str, default="", help="batched workload: block,ctas_per_sm,chunk (default: autotune)")
    p.add_argument("--requests", type=int, default=300, help="served workload: number of requests")
    p.add_argument("--rate", type=float, default=200.0, help="served workload: Poisson arrival rate (1/s)")
    p.add_argument("--plain-instances", type=int, default=0,
                   help="batched workload: instances timed in the plain loop (0 = all)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


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


def cpu_baseline(seconds: float, sc):
    """Oracle port of the reference algorithm on all host cores over a bounded sample."""
    from oracle import oracle
    oracle.build(with_ref=False)
    o = oracle.Oracle("f32")
    rays = sc.num_rays
    cores = os.cpu_count() or 1
    chunk = 1 << 20 if len(sc.elements) < 64 else 1 << 12
    o.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, first_ray=0, count=chunk // 8, nthreads=cores,
            with_ids=False)
    done, first, t0 = 0, 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        o.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, first_ray=first, count=chunk, nthreads=cores,
                with_ids=False)
        done += chunk
        first = (first + chunk) % rays
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": "rays/s", "cores": cores, "kind": "port",
            "sample": f"{done} rays ({done // chunk} chunks of {chunk}) of the {sc.name} workload, "
                      f"{dt:.1f} s, OpenMP over {cores} threads"}


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


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle
    from optixsoltracedemos_gb300 import scenes
    oracle.build(with_ref=False)
    o = oracle.Oracle("f32")
    cores = os.cpu_count() or 1
    # per step: (elements, sun, shape, param, first ray, total rays of that scene or request)
    if args.workload in ("batched", "served"):
        from optixsoltracedemos_gb300 import scenes
        if args.workload == "batched":
            _, poses, suns, counts = batched_workload(args.instances, args.heliostats)
            jobs = [(poses[i], suns[i], scenes.SUN_PILLBOX, 4.65e-3, int(counts[i])) for i in range(len(suns))]
            cfg = {"workload": f"batched_{len(suns)}_instances_large_field_{args.heliostats}_heliostats",
                   "instances": len(suns), "rays_total": int(sum(counts))}
        else:
            _, reqs = served_workload(args.requests, args.rate)
            jobs = [(p, sun, scenes.SUN_PILLBOX, 4.65e-3, rays) for (_, p, sun, rays, _) in reqs]
            cfg = {"workload": "served_requests_fields_3_1000_10000_flat_parabolic", "requests": len(reqs),
                   "rays_total": int(sum(j[4] for j in jobs))}
        sample = 1 << 14  # brute-force closest hit over up to 10,001 elements per ray
        what = f"each step traces {sample} rays of the next instance/request"
    else:
        sc = make_scene(args.workload, args.rays)
        jobs = [(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, sc.num_rays)]
        cfg = config(sc)
        sample = min(1 << 20, sc.num_rays) if args.workload != "large_field" else 1 << 14
        what = f"each step traces {sample} of the {sc.num_rays} rays"

    def step(k):
        el, sun, shape, param, n = jobs[k % len(jobs)]
        o.trace(el, sun, shape, param, first_ray=(k // len(jobs) * sample) % max(1, n), count=sample,
                nthreads=cores, with_ids=False)

    for w in range(args.warmup):
        step(w)
    t0 = time.perf_counter()
    for k in range(args.steps):
        step(k)
    dt = time.perf_counter() - t0
    v = args.steps * sample / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "rays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": cfg,
            "cpu_baseline": {"value": v, "unit": "rays/s", "cores": cores, "kind": "port",
                             "sample": f"{what} (oracle port of the reference algorithm, OpenMP over {cores} "
                                       f"threads)"},
            "e2e": {"value": v, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
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
    from optixsoltracedemos_gb300 import native, scenes
    from optixsoltracedemos_gb300.flux import flux_map_from_hits, flux_l2

    sc = make_scene(args.workload, args.rays)
    N = sc.num_rays
    tr = native.tracer_for(sc, device=local, record_ids=False)
    stream = torch.cuda.Stream(device=local)
    sp = stream.cuda_stream

    for w in range(args.warmup):
        tr.set_seed(w)
        tr.trace_async(sp)
    torch.cuda.synchronize()
    if pg:
        pg.barrier()

    clk = ClockSampler(local)
    clk.start()
    time.sleep(0.3)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for k in range(args.steps):
        tr.set_seed(1000 + k, rank)  # each replica traces its own rays (Philox instance = rank)
        starts[k].record(stream)
        tr.trace_async(sp)
        ends[k].record(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    total_s = e0.elapsed_time(e1) * 1e-3
    launch_s = statistics.mean(s.elapsed_time(e) for s, e in zip(starts, ends)) * 1e-3
    total_s = max_over_ranks(total_s, pg, f"cuda:{local}")
    value = world * N * args.steps / total_s

    # end to end through the C ABI with host buffers
    host = torch.empty(N * 5 * 4, dtype=torch.float32, pin_memory=True)
    elements = sc.elements.copy()
    for _ in range(2):
        tr.set_elements(elements)
        tr.update()
        tr.run_to_host_ptr(host.data_ptr())
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for k in range(args.e2e_steps):
        tr.set_seed(5000 + k, rank)
        tr.set_elements(elements)
        tr.update()
        tr.run_to_host_ptr(host.data_ptr())
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    e2e_s = max_over_ranks(e2e_s, pg, f"cuda:{local}")

    peak, peak_kind = peaks()
    achieved = BYTES_PER_RAY * N / launch_s / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_s / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config(sc),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": NCU_TRAFFIC_PER_LAUNCH if (N == 1 << 24 and sc.name == "single_parabolic") else None,
                     "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": BYTES_PER_RAY * N, "launch_ms": launch_s * 1e3},
        "e2e": {"value": world * N / e2e_s, "unit": "rays/s",
                "h2d_bytes_per_step": int(elements.nbytes + 3 * 8),
                "d2h_bytes_per_step": int(N * BYTES_PER_RAY)},
        "gpu_launches": args.steps,
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_accuracy:
        try:
            from oracle import oracle
            oracle.build(with_ref=False)
            tr.set_seed(0)
            tr.run()
            hits = host.numpy().reshape(N, 5, 4)
            tr.run_to_host(hits.reshape(-1))
            o64 = oracle.Oracle("f64")
            oh, _ = o64.trace(sc.elements, sc.sun_dir, sc.sun_shape, sc.sun_param, count=N, with_ids=False)
            line["flux_l2_vs_fp64"] = flux_l2(flux_map_from_hits(hits, sc.elements[-1], N),
                                              flux_map_from_hits(oh, sc.elements[-1], N))
            del oh
        except Exception as exc:  # accuracy is reported, not required for the timing line
            line["flux_l2_vs_fp64"] = f"unavailable: {exc}"
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.cpu_seconds, sc)
    tr.close()
    if world == 1 and not args.no_systems and args.workload == "single_parabolic" and args.rays is None:
        # the batched and served workloads against the plain per-scene loop (flux maps identical)
        sys_args = argparse.Namespace(**vars(args))
        sys_args.steps, sys_args.warmup = 3, 2
        b = measure_batched(sys_args, local, world)
        line["batched"] = {
            "workload": b["config"]["workload"], "rays": b["config"]["rays_total"],
            "rays_per_s_device": b["value"], "rays_per_s_wall": b["batched_wall_rays_per_s"],
            "rays_per_s_pipelined": b["batched_pipelined_rays_per_s"],
            "plain_loop_rays_per_s": b["plain_loop"]["rays_per_s"], "speedup_vs_plain_loop": b["speedup_vs_plain_loop"],
            "speedup_vs_plain_loop_single_run": b["speedup_vs_plain_loop_single_run"],
            "flux_counts_mismatching_plain": b["plain_loop"]["flux_counts_mismatching_batched"]
            + b["pipelined_flux_counts_mismatching"],
            "tuning_grid": b["config"]["tuning_grid"]}
        v = measure_served(sys_args, local, world)
        line["served"] = {
            "workload": v["config"]["workload"], "requests": v["config"]["requests"], "rays": v["config"]["rays_total"],
            "saturation_rays_per_s": v["served_saturation"]["rays_per_s"],
            "plain_loop_saturation_rays_per_s": v["plain_loop_saturation"]["rays_per_s"],
            "speedup_vs_plain_loop": v["speedup_vs_plain_loop"],
            "poisson_rate_per_s": v["config"]["arrival_rate_per_s"],
            "poisson_p50_s": v["served_poisson"]["p50_s"], "poisson_p99_s": v["served_poisson"]["p99_s"],
            "plain_loop_poisson_p50_s": v["plain_loop_poisson"]["p50_s"],
            "plain_loop_poisson_p99_s": v["plain_loop_poisson"]["p99_s"],
            "flux_counts_mismatching_plain": v["plain_loop_saturation"]["flux_counts_mismatching_served"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()


def batched_workload(n_instances, n_heliostats):
    """The large field at per-instance sun positions with re-aimed heliostats and log-uniform ray
    counts: (base elements, poses per instance, suns, ray counts)."""
    from optixsoltracedemos_gb300 import scenes
    base = scenes.large_field(n_heliostats=n_heliostats, num_rays=1).elements
    suns, counts = scenes.batched_instances(n_instances=n_instances, n_heliostats=n_heliostats)
    poses = [scenes.reaim(base, s) for s in suns]
    return base, poses, suns, counts


def run_batched(args):
    rank, world, local = dist_env()
    line = measure_batched(args, local, world)
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure_batched(args, local, world):
    """Batched workload: one csp_batch run (host element builds, upload, device refit, sun planes,
    one persistent trace launch, flux maps back) against the plain per-scene loop through the
    drop-in handle (per instance: new poses and sun, update, run, device flux map).  Reported three
    ways: device time, wall time of one synchronous run, and the completion interval of pipelined
    runs (run_async / wait: the host builds of a run overlap the device work of the previous one),
    the headline and the `e2e` value."""
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    from optixsoltracedemos_gb300 import build as nbuild
    nbuild.build()
    from optixsoltracedemos_gb300 import native, scenes

    base, poses, suns, counts = batched_workload(args.instances, args.heliostats)
    total = int(counts.sum())
    b = native.Batch(local)
    sid = b.add_scene(base)
    for i in range(len(suns)):
        b.add_instance(sid, suns[i], scenes.SUN_PILLBOX, 4.65e-3, int(counts[i]), seed=0, instance=i, poses=poses[i])
    if args.tuning:
        b.set_tuning(*[int(x) for x in args.tuning.split(",")])
    t0 = time.perf_counter()
    b.run()  # autotune (first run of this scene class) + graph capture
    first_s = time.perf_counter() - t0
    for _ in range(max(0, args.warmup - 1)):
        b.run()
    clk = ClockSampler(local)
    clk.start()
    time.sleep(0.2)
    wall, dev = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        b.run()
        wall.append(time.perf_counter() - t0)
        dev.append(b.timing()[1])
    batch_counts = [b.counts(i).copy() for i in range(len(suns))]
    # pipelined: the host builds of run k + 1 overlap the device work of run k; per-run time =
    # interval between completions
    b.run_async()
    piped = []
    t_prev = None
    for _ in range(args.steps + 1):
        b.run_async()
        b.wait()
        t = time.perf_counter()
        if t_prev is not None:
            piped.append(t - t_prev)
        t_prev = t
    b.wait()
    clocks = clk.stop()
    piped_mismatch = sum(int(not np.array_equal(b.counts(i), batch_counts[i])) for i in range(len(suns)))

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
        tr.set_seed(0, i)
        tr.update()
        tr.run()
        c, _ = tr.flux_map()
        mismatches += int(not np.array_equal(c, batch_counts[i]))
    plain_s = time.perf_counter() - t0
    plain_rays = int(counts[:n_plain].sum())
    tr.close()
    tg, tl = b.tuning(native.GROUP_GRID), b.tuning(native.GROUP_BVH)
    line = {
        "metric": METRIC, "value": total / statistics.median(dev), "unit": "rays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.median(dev) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batched_{len(suns)}_instances_large_field_{args.heliostats}_heliostats",
                   "instances": len(suns), "rays_total": total, "rays_min": int(counts.min()),
                   "rays_max": int(counts.max()), "flux_grid": [100, 100], "sun": "pillbox 4.65 mrad",
                   "slope_error_rad": 1.5e-3, "tuning_grid": tg, "tuning_bvh": tl,
                   "l2_policy": "per-instance scenes and flux maps; no per-ray buffers"},
        "batched_wall_rays_per_s": total / statistics.median(wall),
        "batched_wall_ms": statistics.median(wall) * 1e3,
        "batched_pipelined_rays_per_s": total / statistics.median(piped),
        "batched_pipelined_ms": statistics.median(piped) * 1e3,
        "pipelined_flux_counts_mismatching": piped_mismatch,
        "first_run_s": first_s,
        "plain_loop": {"rays_per_s": plain_rays / plain_s, "instances": n_plain, "seconds": plain_s,
                       "flux_counts_mismatching_batched": mismatches},
        "speedup_vs_plain_loop": (total / statistics.median(piped)) / (plain_rays / plain_s),
        "speedup_vs_plain_loop_single_run": (total / statistics.median(wall)) / (plain_rays / plain_s),
        "e2e": {"value": total / statistics.median(piped), "unit": "rays/s",
                "h2d_bytes_per_step": int(sum(p.nbytes for p in poses)),
                "d2h_bytes_per_step": int(len(suns) * 100 * 100 * 4)},
        "gpu_launches": 1 + 1 + 1,
        "clocks": clocks,
    }
    b.close()
    return line


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


def run_served(args):
    rank, world, local = dist_env()
    line = measure_served(args, local, world)
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure_served(args, local, world):
    """Serving workload through csp_server (continuous batching) against the plain per-scene loop
    (one drop-in handle per scene: update, run, device flux map per request, in arrival order), at
    saturation (all requests queued at once) and with real-time Poisson arrivals."""
    import threading
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    from optixsoltracedemos_gb300 import build as nbuild
    nbuild.build()
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


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "served":
        run_served(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
