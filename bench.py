#!/usr/bin/env python
"""Benchmark of the renderer hot path on one GB300 (or N replicas).

Metric (as named for the reference): Mrays/s of the batched marcher at 20M
points over 256 views of mixed resolution (640x480, 1068x690, 1920x1080;
fx = fy = 0.75 W), beside the plain per-view form, kNN-radii Mqueries/s at
20M points, and forward / forward+backward ms per 1067x690 view on a
1M-point cloud.  All inputs are seeded synthetic scenes of that shape
(renderer_ray_marching_gb300.synthetic); the cloud, index and per-view
records (>= 0.8 GB) exceed the 129 MB L2, so no flush is needed between
timed steps.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

A step is one batched render of all 256 views (value: device-resident
inputs and outputs, CUDA events on the launching stream).  e2e is the same
step through the C ABI with host buffers: the view table goes host->device
and every view's RGBA32F image (colour + depth, the reference's texture
format) comes back to pinned host memory inside the timed region.

--impl reference times the reference's CPU path for the same workload: the
marcher loop of src/ray_marching.cu with an exact 10-NN per step, run by the
oracle's C restatement (the reference tree does not travel to the GPU host)
on all host cores, over a bounded sample of rays per step.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s & kNN-radii Mqueries/s at 20M pts (batched vs plain); fwd+bwd ms/view"
RES = [(640, 480), (1068, 690), (1920, 1080)]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c4"],
                    help="c2: 20M points, 40 boxes, 256 mixed-resolution views (the headline); "
                         "c1: 2M points, 12 boxes, max_radius 0.05, 64 views at 1067x690; "
                         "c4: 100M points, per-surface density log-uniform over 100x, 1024 views at 1067x690, "
                         "fwd+bwd on 64 of them")
    ap.add_argument("--points", type=int, default=None)
    ap.add_argument("--views", type=int, default=None)
    ap.add_argument("--cpu-rays", type=int, default=2_000_000,
                    help="rays per CPU-baseline sample (about 12 s of 16-core CPU work at 20M points)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-views", type=int, default=16,
                    help="views the restated reference GPU path (baseline/ref_gpu) is timed on (0: skip)")
    # switches for short profiling runs (never used for a reported number)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-fwdbwd", action="store_true")
    ap.add_argument("--resolution", default=None, help="WxH for every view instead of the mixed set")
    return ap.parse_args()


T0 = time.perf_counter()


def log(msg):
    print("[bench %7.1fs] %s" % (time.perf_counter() - T0, msg), file=sys.stderr, flush=True)


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


WORKLOADS = {
    # points, boxes, per-surface density range, views, resolutions (None: the
    # reference's README intrinsics, 1067x690), max_radius (the -r flag)
    "c1": dict(points=2_000_000, boxes=12, density=1.0, views=64, res=None, max_radius=0.05),
    "c2": dict(points=20_000_000, boxes=40, density=1.0, views=256, res=RES, max_radius=0.1),
    "c4": dict(points=100_000_000, boxes=12, density=100.0, views=1024, res=None, max_radius=0.1),
}


def workload_spec(args):
    w = dict(WORKLOADS[getattr(args, "workload", "c2")])
    if getattr(args, "points", None):
        w["points"] = args.points
    if getattr(args, "views", None):
        w["views"] = args.views
    if getattr(args, "resolution", None):
        ww, hh = (int(x) for x in args.resolution.lower().split("x"))
        w["res"] = [(ww, hh)]
    return w


def workload(args, rank):
    from renderer_ray_marching_gb300 import synthetic as syn, views_from_specs
    w = workload_spec(args)
    sc = syn.make_scene(w["points"], n_boxes=w["boxes"], seed=2000 + rank, density_range=w["density"])
    specs = syn.make_views(w["views"], seed=3000 + rank, boxes=sc.boxes, resolutions=w["res"])
    return sc, views_from_specs(specs)


def workload_name(args, n_points, n_views):
    w = workload_spec(args)
    if w["res"] is None:
        shape = "%d views at 1067x690 (fx=803.8)" % n_views
    else:
        shape = "%d views (%s, fx=0.75W)" % (n_views, "/".join("%dx%d" % r for r in w["res"]))
    dens = "" if w["density"] <= 1.0 else ", per-surface density log-uniform over %gx" % w["density"]
    return "batched render of %s over a %d-point synthetic room, %d boxes%s, max_radius %g" % (
        shape, n_points, w["boxes"], dens, w["max_radius"])


class Clocks:
    """nvidia-smi sampled every 200 ms while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def capture_figures(name):
    """Figures of a committed ncu summary (profiles/<name>.json: DRAM bytes
    per unit, issue and occupancy counters), or None."""
    p = os.path.join(ROOT, "profiles", name + ".json")
    if os.path.exists(p):
        return json.load(open(p))
    return None


def hit_checksum(keep) -> int:
    """Order-sensitive 64-bit checksum of every view's hit map (full-size
    property checks: the same batch through another path must give the same
    hit indices)."""
    import torch
    total = 0
    for i, (_, h) in enumerate(keep):
        flat = h.reshape(-1).to(torch.int64)
        w = torch.arange(1, flat.numel() + 1, device=flat.device, dtype=torch.int64) * (2 * i + 1)
        total = (total * 1000003 + int(((flat + 2) * w).sum().item())) & 0xFFFFFFFFFFFFFFFF
    return total


def sample_pixels(views, n_rays, seed):
    """A bounded, seeded sample of pixels spread evenly over the views
    (sorted linear indices per view)."""
    rng = np.random.default_rng(seed)
    per = max(1, n_rays // len(views))
    return [np.sort(rng.choice(v.pixels, min(per, v.pixels), replace=False)).astype(np.int64) for v in views]


def cpu_sample_render(ix, views, panes, radii_clamped, pixels, threads=0):
    """Oracle (the reference marcher loop restated in C, exact 10-NN per
    step) over the sampled pixels of each view, each view with the pane
    distance the device evaluates.  Returns (seconds, [(hit, depth, steps)])."""
    import oracle
    jobs = [(oracle.make_view(v.cam2world, v.width, v.height, float(p)), pix)
            for v, p, pix in zip(views, panes, pixels)]
    t0 = time.perf_counter()
    outs = [ix.render(radii_clamped, ov, pix, threads=threads) for ov, pix in jobs]
    return time.perf_counter() - t0, outs


def compare_with_oracle(gpu, cpu):
    """Counts of disagreements between the GPU frames and the oracle on the
    sampled pixels: hit index, depth bits, step count where the ray hits,
    and misses that the GPU marched longer than the oracle (exit culling
    may only shorten a miss)."""
    c = {"rays": 0, "hit_mismatch": 0, "depth_bit_mismatch": 0, "step_mismatch_on_hits": 0,
         "miss_steps_above_oracle": 0}
    for (gh, gd, gs), (oh, od, os_) in zip(gpu, cpu):
        c["rays"] += int(oh.size)
        c["hit_mismatch"] += int((gh != oh).sum())
        c["depth_bit_mismatch"] += int((gd.view(np.int32) != od.view(np.int32)).sum())
        h = oh >= 0
        c["step_mismatch_on_hits"] += int((gs[h] != os_[h]).sum())
        c["miss_steps_above_oracle"] += int((gs[~h] > os_[~h]).sum())
    return c


def time_ref_gpu(sc, views, keep, max_radius, dev):
    """The reference's GPU path, restated (baseline/ref_gpu: FLANN's CUDA
    kd-tree and the reference's render kernel, one view per launch, 16x16
    blocks, per-pixel global result arrays), timed per view with CUDA events
    over the given views; its hit maps are compared with the library's for
    the same views.  Also its radii search kernel and, sampled, the
    reference's host sqrt loop over device elements."""
    import torch
    from baseline.ref_gpu import RefGpu
    t0 = time.perf_counter()
    rg = RefGpu(sc.xyz)
    tb = time.perf_counter() - t0
    _, _, radii_ms = rg.radii(max_radius)
    loop_s = rg.sqrt_loop_seconds_per_point(20000)
    npix = max(v.pixels for v in views)
    hit = torch.empty(npix, dtype=torch.int32, device=dev)
    depth = torch.empty(npix, dtype=torch.float32, device=dev)
    rg.render_into(views[0].cam2world, views[0].width, views[0].height, views[0].fov, hit.data_ptr(),
                   depth.data_ptr())  # warm-up
    ms, rays, mismatch = 0.0, 0, 0
    for v, (_, lib_hit) in zip(views, keep):
        ms += rg.render_into(v.cam2world, v.width, v.height, v.fov, hit.data_ptr(), depth.data_ptr())
        rays += v.pixels
        mismatch += int((hit[:v.pixels] != lib_hit.reshape(-1)).sum().item())
    n = int(sc.xyz.shape[0])
    rg.close()
    return {"mrays_s": round(rays / (ms * 1e-3) / 1e6, 4), "views": len(views), "rays": int(rays),
            "ms": round(ms, 2), "hit_mismatch_vs_library": mismatch,
            "radii_search_ms": round(radii_ms, 3), "radii_search_mqueries_s": round(n / (radii_ms * 1e-3) / 1e6, 2),
            "radii_host_sqrt_loop_s_per_point": loop_s,
            "radii_as_shipped_s": round(radii_ms * 1e-3 + loop_s * n, 2),
            "tree_build_host_s": round(tb, 2),
            "what": "baseline/ref_gpu: the reference's render kernel and FLANN CUDA kd-tree restated, one view "
                    "per launch; radii_as_shipped adds the reference's host sqrt loop (main.cu:110-112) "
                    "timed on 20,000 points and scaled"}


def cpu_radii(sc, threads):
    """The reference's radii precompute on the host cores (the oracle's
    exact 2-NN, build and query both timed).  Returns (seconds, build
    seconds)."""
    import oracle
    t0 = time.perf_counter()
    ix = oracle.Index(sc.xyz)
    tb = time.perf_counter() - t0
    ix.radii(0.0, threads=threads)
    return time.perf_counter() - t0, tb, ix


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    import oracle
    from renderer_ray_marching_gb300 import synthetic as syn  # noqa: F401
    sc, views = workload(args, 0)
    ix = oracle.Index(sc.xyz)
    radii, _ = ix.radii(workload_spec(args)["max_radius"])
    # the pane of each view as the reference evaluates it (device tanf); on
    # the CPU path the host tanf stands in
    import math
    vp = [(v, np.float32(np.float32(v.width) / (np.float32(2.0) * np.float32(math.tan(np.float32(0.5) * np.float32(v.fov))))))
          for v in views]
    cores = os.cpu_count() or 1
    rng_seed = 99
    times = []
    rays_per = 0
    n_rays = args.cpu_rays
    for step in range(args.warmup + args.steps):
        rng = np.random.default_rng(rng_seed + step)
        per = max(1, n_rays // len(vp))
        t0 = time.perf_counter()
        rays = 0
        for v, pane in vp:
            pix = rng.choice(v.pixels, min(per, v.pixels), replace=False).astype(np.int64)
            ix.render(radii, oracle.make_view(v.cam2world, v.width, v.height, float(pane)), pix, threads=cores)
            rays += pix.shape[0]
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
            rays_per = rays
    value = rays_per / float(np.mean(times)) / 1e6
    sample = "%d rays per step spread over %d views (%d points), exact 10-NN per march step" % (
        rays_per, len(vp), sc.xyz.shape[0])
    line = {"metric": METRIC, "value": round(value, 4), "unit": "Mrays/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * float(np.mean(times)), 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_name(args, sc.xyz.shape[0], len(vp)), "points": int(sc.xyz.shape[0]),
                       "views": len(vp)},
            "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    from renderer_ray_marching_gb300 import Renderer, _abi

    ws, rank, local = dist_info()
    dist = ws > 1
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda:%d" % local)
    stream = torch.cuda.Stream(device=dev)
    max_radius = float(workload_spec(args)["max_radius"])

    sc, views = workload(args, rank)
    log("workload ready: %d points, %d views" % (sc.xyz.shape[0], len(views)))
    xyz_d = torch.from_numpy(sc.xyz).to(dev)
    rgb_d = torch.from_numpy(sc.rgb).to(dev)
    torch.cuda.synchronize()

    with torch.cuda.stream(stream):
        r = Renderer(leaf_size=16, device=local, stream=stream.cuda_stream)

        # ---- radii: upload from device memory, index build, radii kernel
        rad_d = torch.empty(sc.xyz.shape[0], dtype=torch.float32, device=dev)
        nn_d = torch.empty(sc.xyz.shape[0], dtype=torch.int32, device=dev)
        radii_ms, build_ms, query_ms = [], [], []
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        em = torch.cuda.Event(enable_timing=True)
        for i in range(args.warmup + 2):
            e0.record(stream)
            r.set_cloud(xyz_d, rgb_d)
            r.build_index()
            em.record(stream)
            r._check(r._lib.rm_radii_compute(r._h, max_radius, rad_d.data_ptr(), nn_d.data_ptr(), _abi.RM_DEVICE))
            e1.record(stream)
            e1.synchronize()
            if i >= args.warmup:
                radii_ms.append(e0.elapsed_time(e1))
                build_ms.append(e0.elapsed_time(em))
                query_ms.append(em.elapsed_time(e1))
        radii_mq = sc.xyz.shape[0] / (float(np.median(radii_ms)) * 1e-3) / 1e6
        log("radii %.2f ms (upload+build %.2f, query %.2f)" % (float(np.median(radii_ms)), float(np.median(build_ms)),
                                                             float(np.median(query_ms))))

        # ---- autotune on a subset of views
        tune = r.get_launch() if args.no_autotune else r.autotune(views[:32])
        log("launch %s" % tune)

        # ---- batched, device-resident
        frames = (_abi.RmFrame * len(views))()
        keep = []
        for i, v in enumerate(views):
            rgbd = torch.empty((v.height, v.width, 4), dtype=torch.float32, device=dev)
            hit = torch.empty((v.height, v.width), dtype=torch.int32, device=dev)
            frames[i].rgbd = rgbd.data_ptr()
            frames[i].hit = hit.data_ptr()
            keep.append((rgbd, hit))
        cviews = (_abi.RmView * len(views))(*[v.to_c() for v in views])
        total_rays = sum(v.pixels for v in views)
        for _ in range(args.warmup):
            r.render_batch_into(views, frames, device=True, cviews=cviews)
            r.synchronize()
            log("warm-up batch %s" % r.stats())
        r.synchronize()
        if dist:
            tdist.barrier()
        torch.cuda.synchronize()
        clocks = Clocks(local)
        clocks.start()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        kern_ms, steps_total, st = [], 0, {}
        for k in range(args.steps):
            starts[k].record(stream)
            r.render_batch_into(views, frames, device=True, cviews=cviews)
            ends[k].record(stream)
            st = r.stats()  # synchronises; kernel time from events inside the graph
            kern_ms.append(st["kernel_ms"])
            steps_total = st["steps"]
        torch.cuda.synchronize()
        clk = clocks.stop()
        step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
        t_step = float(np.mean(step_ms))
        if dist:
            tt = torch.tensor([t_step], device=dev)
            tdist.all_reduce(tt, op=tdist.ReduceOp.MAX)
            t_step = float(tt.item())
        value = ws * total_rays / (t_step * 1e-3) / 1e6
        hits_total = int(sum(int((h >= 0).sum().item()) for _, h in keep))
        hit_sum = hit_checksum(keep)
        walk = {"leaves_per_warp_step": round(st["packet_leaves"] / max(st["warp_steps"], 1), 2),
                "nodes_per_warp_step": round(st["packet_nodes"] / max(st["warp_steps"], 1), 2),
                "lane_steps_per_warp_step": round(st["packet_steps"] / max(st["warp_steps"], 1), 2),
                "queue_spills": st["queue_spills"], "dfs_walks": st["dfs_walks"],
                "search_errors": st["search_errors"]}
        checks = {}

        # ---- the same batch again with per-pixel step counts: its hit maps
        # must equal the timed ones, and a seeded pixel sample of it is
        # compared with the oracle below
        sample = None
        if rank == 0 and not args.no_cpu_baseline:
            steps_bufs = []
            for i, v in enumerate(views):
                sb = torch.empty((v.height, v.width), dtype=torch.int32, device=dev)
                frames[i].steps = sb.data_ptr()
                steps_bufs.append(sb)
            r.render_batch_into(views, frames, device=True, cviews=cviews)
            r.synchronize()
            checks["verify_render_equals_timed"] = hit_checksum(keep) == hit_sum
            pixels = sample_pixels(views, args.cpu_rays, 7)
            gpu_sample = []
            for (rgbd, hit), sb, pix in zip(keep, steps_bufs, pixels):
                ip = torch.from_numpy(pix).to(dev)
                gpu_sample.append((hit.reshape(-1)[ip].cpu().numpy(), rgbd.reshape(-1, 4)[ip, 3].cpu().numpy(),
                                   sb.reshape(-1)[ip].cpu().numpy()))
            for i in range(len(views)):
                frames[i].steps = None
            del steps_bufs
            sample = (pixels, gpu_sample, r.view_pane(views))

        # ---- the same batch with one independent tree walk per ray (the
        # reference's execution model) instead of the warp packet walk
        per_ray = None
        if not args.skip_plain:
            L0 = r.get_launch()
            r.set_launch(L0["tile_w"], L0["tile_h"], 1, 4, 0)
            r.render_batch_into(views, frames, device=True, cviews=cviews)
            r.synchronize()
            e0.record(stream)
            r.render_batch_into(views, frames, device=True, cviews=cviews)
            e1.record(stream)
            e1.synchronize()
            per_ray = total_rays / (e0.elapsed_time(e1) * 1e-3) / 1e6
            checks["per_ray_equals_packet"] = hit_checksum(keep) == hit_sum
            r.set_launch(L0["tile_w"], L0["tile_h"], L0["rays_per_lane"], L0["ctas_per_sm"], L0["search"])
            log("per-ray walk %.2f Mrays/s" % per_ray)

        # ---- plain per-view form, same views
        plain, plain_ms = None, None
        if not args.skip_plain:
            r.synchronize()
            e0.record(stream)
            for i, v in enumerate(views):
                r._check(r._lib.rm_render(r._h, ctypes.byref(cviews[i]), ctypes.byref(frames[i]), _abi.RM_DEVICE))
            e1.record(stream)
            e1.synchronize()
            plain_ms = e0.elapsed_time(e1)
            checks["plain_equals_batched"] = hit_checksum(keep) == hit_sum
            plain = total_rays / (plain_ms * 1e-3) / 1e6
        log("timed batch %.1f ms/step, plain %s ms" % (t_step, plain_ms))

        # ---- the reference's GPU path, restated, on the first views
        ref_gpu = None
        if args.ref_views > 0:
            ref_gpu = time_ref_gpu(sc, views[:args.ref_views], keep[:args.ref_views], max_radius, dev)
            log("reference GPU path %s" % ref_gpu)

        # ---- e2e: host buffers through the C ABI (views in, RGBA32F images out)
        e2e, h2d, d2h = None, 0, 0
        if not args.skip_e2e:
            del keep, frames
            torch.cuda.empty_cache()
            host_frames = (_abi.RmFrame * len(views))()
            host_keep = []
            for i, v in enumerate(views):
                b = torch.empty((v.height, v.width, 4), dtype=torch.float32).pin_memory()
                host_frames[i].rgbd = b.data_ptr()
                host_keep.append(b)
            r.render_batch_into(views, host_frames, device=False, cviews=cviews)
            e2e_t = []
            for _ in range(max(2, args.steps // 2)):
                t0 = time.perf_counter()
                r.render_batch_into(views, host_frames, device=False, cviews=cviews)
                e2e_t.append(time.perf_counter() - t0)
            e2e = total_rays / float(np.mean(e2e_t)) / 1e6
            h2d = len(views) * ctypes.sizeof(_abi.RmView)
            d2h = total_rays * 16
            log("e2e %.1f ms (last call's batched launch %.1f ms on the device)" % (
                1e3 * float(np.mean(e2e_t)), r.stats()["kernel_ms"]))
            del host_keep

        # ---- forward / forward+backward per 1067x690 view on a 1M-point cloud
        fb = {"fwd_ms": None, "fwdbwd_ms": None, "ratio": None}
        if not args.skip_fwdbwd:
            if args.workload == "c4":
                fb = fwd_bwd(args, dev, stream, rank, scene=sc, views=views[:64])
            else:
                fb = fwd_bwd(args, dev, stream, rank)
            log("fwd/bwd %s" % fb)
        r.close()

    peak, peak_kind = measured_peak()
    kms = float(np.median(kern_ms))
    alg_bytes = 20 * total_rays + 16 * hits_total + 160 * steps_total
    achieved = alg_bytes / (kms * 1e-3) / 1e9
    mc = capture_figures("march_batch_traffic") or {}
    traffic = int(mc["dram_bytes_per_ray"] * total_rays) if "dram_bytes_per_ray" in mc else None
    n_pts = int(sc.xyz.shape[0])
    radii_s = float(np.median(radii_ms)) * 1e-3
    rc = capture_figures("radii_traffic") or {}
    radii_roof = {"bound": "hbm", "kernel": "index build + k_radii_packet",
                  "achieved": round(136 * n_pts / radii_s / 1e9, 1), "peak": peak, "unit": "GB/s",
                  "frac": round(136 * n_pts / radii_s / 1e9 / peak, 4),
                  "bytes_model": "136 B/point: 16 B point read, 64 B radix sort, 32 B record gather, "
                                 "16 B query read, 8 B radius + neighbour write",
                  "traffic": int(rc["dram_bytes_per_query"] * n_pts) if "dram_bytes_per_query" in rc else None,
                  "dram_bytes_per_query": rc.get("dram_bytes_per_query"),
                  "query_issue_active_pct": rc.get("sm_issue_active_pct")}
    out = {"metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(t_step, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": workload_name(args, n_pts, len(views)),
                      "points": n_pts, "views": len(views), "rays_per_step": int(total_rays),
                      "max_radius": max_radius,
                      "l2": "inputs larger than L2 (cloud + index >= 0.8 GB), no flush",
                      "launch": tune, "parallelism": "replicas" if ws > 1 else "single"},
           "plain_mrays_s": None if plain is None else round(plain, 3),
           "per_ray_walk_mrays_s": None if per_ray is None else round(per_ray, 3),
           "batched_over_plain": None if plain is None else round(value / ws / plain, 3),
           "ref_gpu_path": ref_gpu,
           "batched_over_ref_gpu": None if ref_gpu is None else round(value / ws / ref_gpu["mrays_s"], 2),
           "radii_mqueries_s": round(radii_mq, 3), "radii_ms": round(float(np.median(radii_ms)), 3),
           "radii_build_ms": round(float(np.median(build_ms)), 3), "radii_query_ms": round(float(np.median(query_ms)), 3),
           "fwd_ms_per_view": fb["fwd_ms"], "fwdbwd_ms_per_view": fb["fwdbwd_ms"],
           "fwdbwd_over_fwd": fb["ratio"],
           "steps_per_ray": round(steps_total / total_rays, 3), "hit_fraction": round(hits_total / total_rays, 4),
           "walk": walk,
           "checks": checks,
           "e2e": {"value": None if e2e is None else round(e2e, 3), "unit": "Mrays/s", "h2d_bytes_per_step": int(h2d),
                   "d2h_bytes_per_step": int(d2h)},
           "roofline": {"bound": "hbm", "kernel": "k_march_batch", "achieved": round(achieved, 1), "peak": peak,
                        "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                        "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                        "bytes_model": "20 B out + 16 B colour per hit + 160 B per distance step (10 float4 candidates)",
                        "kernel_ms": round(kms, 3),
                        "binding_bound": "instruction issue (the index is L2-resident); figures below from the "
                                         "committed capture " + str(mc.get("source")),
                        "sm_issue_active_pct": mc.get("sm_issue_active_pct"),
                        "eligible_warps_per_scheduler": mc.get("eligible_warps_per_scheduler"),
                        "warp_inst_per_lane_step": mc.get("warp_inst_per_lane_step"),
                        "warp_inst_per_warp_step": mc.get("warp_inst_per_warp_step"),
                        "l2_hit_pct": mc.get("l2_hit_pct")},
           "roofline_radii": radii_roof,
           "clocks": clk,
           "gpu_launches": 2 * args.steps}
    if sample is not None:
        cores = os.cpu_count() or 1
        pixels, gpu_sample, panes = sample
        rad_h = np.minimum(rad_d.cpu().numpy(), np.float32(max_radius))
        t0 = time.perf_counter()
        import oracle
        ix = oracle.Index(sc.xyz)
        tb = time.perf_counter() - t0
        secs, cpu_out = cpu_sample_render(ix, views, panes, rad_h, pixels, threads=cores)
        rays = int(sum(p.size for p in pixels))
        log("cpu baseline %d rays %.1f s (build %.1f s)" % (rays, secs, tb))
        checks["oracle_sample"] = compare_with_oracle(gpu_sample, cpu_out)
        log("oracle sample %s" % checks["oracle_sample"])
        out["cpu_baseline"] = {"value": round(rays / secs / 1e6, 5), "unit": "Mrays/s", "cores": cores,
                               "kind": "port",
                               "sample": "%d rays (%d per view over %d views), oracle kd-tree (build %.1f s, not "
                                         "timed); the same pixels are compared with the GPU frames" % (
                                             rays, pixels[0].size, len(views), tb)}
        del ix
        rsecs, rbuild, _ = cpu_radii(sc, cores)
        log("cpu radii %.1f s (build %.1f s)" % (rsecs, rbuild))
        out["cpu_baseline_radii"] = {"value": round(n_pts / rsecs / 1e6, 4), "unit": "Mqueries/s", "cores": cores,
                                     "kind": "port",
                                     "sample": "all %d points: oracle kd-tree build + exact self-inclusive 2-NN, "
                                               "both timed (build %.1f s)" % (n_pts, rbuild)}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist:
        tdist.destroy_process_group()


def fwd_bwd(args, dev, stream, rank, scene=None, views=None):
    """Forward (plain render) and forward + loss gradient + backward per view:
    by default 16 1067x690 views of a 1M-point cloud; or the given scene and
    views.  Targets come from a copy with xyz + N(0, 5 mm) and colour +-30."""
    import torch
    from renderer_ray_marching_gb300 import Renderer, _abi, synthetic as syn, views_from_specs
    sc = scene if scene is not None else syn.make_scene(1_000_000, n_boxes=12, seed=4000 + rank)
    if views is None:
        views = views_from_specs(syn.make_views(16, seed=4100 + rank, boxes=sc.boxes))
    rng = np.random.default_rng(5)
    xt = (sc.xyz + rng.normal(0, 0.005, sc.xyz.shape)).astype(np.float32)
    ct = np.clip(sc.rgb.astype(np.int32) + rng.integers(-30, 31, sc.rgb.shape), 0, 255).astype(np.uint8)
    r = Renderer(device=dev.index, stream=stream.cuda_stream)
    rt = Renderer(device=dev.index, stream=stream.cuda_stream)
    for rr, x, c in ((r, sc.xyz, sc.rgb), (rt, xt, ct)):
        rr.set_cloud(x, c)
        rr.build_index()
        rr.compute_radii(0.1)  # -r default (main.cu:70)
    n = sc.xyz.shape[0]
    tg = [rt.render(v, outputs=("rgbd", "hit"), device=True) for v in views]
    rt.close()
    g = [torch.zeros((n, 3), device=dev), torch.zeros((n, 3), device=dev), torch.zeros(n, device=dev)]
    frames = [{"rgbd": torch.empty((v.height, v.width, 4), device=dev),
               "hit": torch.empty((v.height, v.width), dtype=torch.int32, device=dev)} for v in views]
    dl_rgb = [torch.empty((v.pixels, 3), device=dev) for v in views]
    dl_d = [torch.empty(v.pixels, device=dev) for v in views]
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]

    def fwd(i):
        r.render_into(views[i], frames[i], device=True)

    def bwd(i):
        f, t = frames[i], tg[i]
        both = (f["hit"] >= 0) & (t["hit"] >= 0)
        d = (f["rgbd"] - t["rgbd"]).reshape(-1, 4)
        m = both.reshape(-1, 1).float()
        torch.mul(d[:, :3], 2.0 * m, out=dl_rgb[i])
        torch.mul(torch.sign(d[:, 3]), m[:, 0], out=dl_d[i])
        r._check(r._lib.rm_backward(r._h, ctypes.byref(views[i].to_c()), 1, dl_rgb[i].data_ptr(),
                                    dl_d[i].data_ptr(), f["hit"].data_ptr(), g[0].data_ptr(),
                                    g[1].data_ptr(), g[2].data_ptr(), _abi.RM_DEVICE))

    for i in range(len(views)):  # warm-up
        fwd(i)
        bwd(i)
    torch.cuda.synchronize()
    e[0].record(stream)
    for i in range(len(views)):
        fwd(i)
    e[1].record(stream)
    for i in range(len(views)):
        fwd(i)
        bwd(i)
    e[2].record(stream)
    e[2].synchronize()
    f_ms = e[0].elapsed_time(e[1]) / len(views)
    fb_ms = e[1].elapsed_time(e[2]) / len(views)
    r.close()
    return {"fwd_ms": round(f_ms, 3), "fwdbwd_ms": round(fb_ms, 3), "ratio": round(fb_ms / f_ms, 3)}


if __name__ == "__main__":
    main()
