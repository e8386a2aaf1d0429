"""Benchmark of the ray--bicubic-patch path on GB300.

Workload (one step = one frame): the seeded displaced torus (R=4, r=1,
128x128 = 16,384 bicubic patches, radial displacement sigma 0.05 on interior
control points), 1920x1080 primary rays plus one mirror bounce, Cook-Torrance
PBR with two point lights and their shadow rays, Bezier clipping at the
reference tolerance 2^-12 in FP32 followed by the FP64 Newton polish of every
hit (so the metric's <= 1e-5 relative t error holds; it is verified on a seeded
1% pixel subset against the FP64 oracle outside the timed region).

value  = total rays (primary + bounce + shadow) / device time of K frames, scene
         resident in HBM, L2 flushed before every frame.
e2e    = the same through cgs_render_host (host framebuffer, copies inside the
         timed region).
--impl reference: the reference's CPU path (oracle/_ref if the reference
         compiled, else the oracle's restatement) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W, H = 1920, 1080
DEPTH = 1
L2_BYTES = 129 * 1024 * 1024
FP32_FLOPS_PER_CLK_SM = 256  # 128 FP32 lanes x FMA
SMS = 152


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--schedule", default="wavefront", choices=["wavefront", "plain"])
    ap.add_argument("--precision", default="polish64", choices=["fp32", "polish64"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--quick", action="store_true", help="no plain-path comparison, no FP64 check")
    ap.add_argument("--size", default=None, help="WxH of a smaller frame (profiling cases); default 1920x1080")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
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
        import statistics
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = max(mx, float(p[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def traffic_summary():
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary, if any."""
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_traffic.json")) as f:
            return json.load(f)
    except Exception:
        return None


def cpu_leg(scene, camera, sample_rows=1):
    import oracle
    o = oracle.OracleScene(scene)
    r = o.render_rows(camera, W, H, 0, sample_rows, depth=DEPTH)
    rays = r["primary"] + r["bounce"] + r["shadow"]
    return {"value": rays / r["seconds"] / 1e6, "unit": "Mrays/s", "cores": r["threads"], "kind": "port",
            "sample": f"every {sample_rows} row(s) of the {W}x{H} frame: {r['primary']} primary + {r['bounce']} "
                      f"bounce + {r['shadow']} shadow rays in {r['seconds']:.2f} s (oracle restatement, "
                      f"{r['threads']} threads, 32x32 tiles)",
            "seconds": r["seconds"], "rays": rays}


def reference_cpu_leg(scene, camera, rows):
    """The reference's own CPU tracer when it compiled here (oracle/_ref), else the restatement."""
    try:
        from oracle import ref as R
        if R.available():
            res = R.render_rows(scene, camera, W, H, 0, rows, depth=DEPTH)
            rays = res["primary"] + res["bounce"] + res["shadow"]
            return {"value": rays / res["seconds"] / 1e6, "unit": "Mrays/s", "cores": res["threads"],
                    "kind": "reference", "sample": f"every {rows} row(s) of the {W}x{H} frame, reference "
                                                   f"CPURayTracer compiled from its own sources",
                    "seconds": res["seconds"], "rays": rays}
    except Exception:
        pass
    return cpu_leg(scene, camera, rows)


def run_reference(args, rank, world):
    from cgspline_gb300 import scenes
    if rank != 0:
        return
    scene, cam = scenes.scene_c2(), scenes.camera_c2()
    rows = 2
    for _ in range(args.warmup):
        reference_cpu_leg(scene, cam, rows * 4)
    tot_rays, tot_s, leg = 0, 0.0, None
    for _ in range(args.steps):
        leg = reference_cpu_leg(scene, cam, rows)
        tot_rays += leg["rays"]
        tot_s += leg["seconds"]
    v = tot_rays / tot_s / 1e6
    line = {"metric": "Mrays/s at <=1e-5 rel-t err vs FP64 (C2 torus 1080p + 1 bounce, PBR)", "value": v,
            "unit": "Mrays/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tot_s / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded displaced torus)", "impl": "reference",
            "config": {"workload": f"torus 16384 patches, {W}x{H} primary + {DEPTH} bounce, PBR, 2 point lights, "
                                   f"CPU sample = every {rows} rows"},
            "cpu_baseline": {k: leg[k] for k in ("kind", "cores", "sample")} | {"value": v, "unit": "Mrays/s"},
            "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    global W, H
    if args.size:
        W, H = (int(x) for x in args.size.lower().split("x"))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import numpy as np
    import torch

    from cgspline_gb300 import rt, scenes

    dist = world > 1
    if dist:
        import torch.distributed as td
        td.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    scene, cam = scenes.scene_c2(), scenes.camera_c2()
    g = rt.GpuScene(scene, device=local)
    sched = rt.WAVEFRONT if args.schedule == "wavefront" else rt.PLAIN
    prec = rt.FP32_POLISH64 if args.precision == "polish64" else rt.FP32
    tracer = rt.RayTracer(rt.Options(recursion_depth=DEPTH, precision=prec, schedule=sched))
    frame = rt.Frame(W, H, alignment=32, device=local)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def step():
        # a scene refuses a new render while its previous one is in flight
        # (src/rt/RayTracer.cu:110-116), so frames are issued one at a time;
        # the events below time each frame on the device.
        tracer.render(frame, cam, g, stream)

    for _ in range(max(3, args.warmup)):
        step()
        torch.cuda.synchronize()
    counters = g.counters()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        td.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.fill_(float(k))  # L2 flush: 2x L2 bytes written between frames
            starts[k].record(stream)
            step()
            ends[k].record(stream)
            ends[k].synchronize()
        torch.cuda.synchronize()
    ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = float(sum(ms))
    if dist:
        t = torch.tensor([total_ms], device=dev)
        td.all_reduce(t, op=td.ReduceOp.MAX)
        total_ms = float(t.item())
    rays_per_frame = counters["rays"]
    value = rays_per_frame * args.steps * world / (total_ms * 1e-3) / 1e6

    # e2e: the C-ABI host entry point (framebuffer copied to host inside the timed region)
    fb_host = None
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fb_host, _ = tracer.render_host(cam, g, W, H, linear=False)
    e2e_s = time.perf_counter() - t0
    e2e = {"value": rays_per_frame * args.steps / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": 44,
           "d2h_bytes_per_step": W * H * 4}

    extra = {}
    if not args.quick and rank == 0:
        # dominant-kernel roofline from the kernel's own work counters
        c = counters
        nrays, nodes, hashes, cand, iters = c["rays"], c["nodes"], c["hash_lookups"], c["candidates"], c["iterations"]
        alg_bytes = 48 * nrays + 64 * nodes + 8 * hashes + 320 * cand
        alg_flops = 12 * nodes + 296 * cand + 470 * iters + 200 * nrays
        sec_per_frame = total_ms / args.steps / 1e3
        peaks, pk = measured_peaks()
        clocks_now = clk.summary()
        mhz = clocks_now["sm_mhz"] or 2070.0
        fp32_peak = SMS * FP32_FLOPS_PER_CLK_SM * mhz * 1e6 / 1e12
        achieved = alg_bytes / sec_per_frame / 1e9
        tr = traffic_summary()
        extra["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                             "frac": achieved / peaks["hbm_gbs"], "traffic": tr.get("bytes_per_frame") if tr else None,
                             "peak_source": pk, "kernel": "whole frame (closest + shade + shadow + resolve)",
                             "fp32": {"achieved": alg_flops / sec_per_frame / 1e12, "peak": fp32_peak,
                                      "unit": "TFLOP/s", "frac": alg_flops / sec_per_frame / 1e12 / fp32_peak,
                                      "peak_source": f"nominal 152 SM x 256 flop/clk at {mhz:.0f} MHz"},
                             "per_ray": {"nodes": nodes / nrays, "hash_lookups": hashes / nrays,
                                         "candidates": cand / nrays, "clip_iterations": iters / nrays}}
        # plain per-frame GPU path (one thread per pixel megakernel)
        if sched != rt.PLAIN:
            plain = rt.RayTracer(rt.Options(recursion_depth=DEPTH, precision=prec, schedule=rt.PLAIN))
            for _ in range(2):
                plain.render(frame, cam, g, stream)
                torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            pm = 0.0
            for k in range(3):
                flush.fill_(float(k))
                e0.record(stream)
                plain.render(frame, cam, g, stream)
                e1.record(stream)
                torch.cuda.synchronize()
                pm += e0.elapsed_time(e1)
            extra["plain_path"] = {"value": rays_per_frame * 3 / (pm * 1e-3) / 1e6, "unit": "Mrays/s",
                                   "ms_per_step": pm / 3}
        # accuracy vs FP64 on a seeded 1% pixel subset of the primary rays
        import oracle
        o = oracle.OracleScene(scene)
        allr = oracle.camera_rays(cam, W, H)
        sub = scenes.random_subset(W * H, 0.01, seed=77)
        rays = np.ascontiguousarray(allr[:, sub])
        o64 = o.intersect(rays, precision=oracle.FP64)
        gg = g.intersect(torch.from_numpy(rays).to(dev), precision=prec)
        gp, gt = gg["patch"].cpu().numpy(), gg["t"].cpu().numpy()
        hm = float(((gp >= 0) != (o64["patch"] >= 0)).mean())
        both = (gp >= 0) & (o64["patch"] >= 0)
        rel = np.abs(gt[both] - o64["t"][both]) / o64["t"][both]
        extra["accuracy"] = {"subset_rays": int(sub.size), "max_rel_t_err": float(rel.max(initial=0.0)),
                             "hit_miss_disagreement": hm,
                             "patch_disagreement": float((both & (gp != o64["patch"])).mean())}
    if not args.no_cpu and rank == 0 and world == 1:
        extra["cpu_baseline"] = {k: v for k, v in cpu_leg(scene, cam, 1).items() if k not in ("seconds", "rays")}
    if rank == 0:
        line = {"metric": "Mrays/s at <=1e-5 rel-t err vs FP64 (C2 torus 1080p + 1 bounce, PBR)", "value": value,
                "unit": "Mrays/s", "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
                "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32+f64polish" if prec == rt.FP32_POLISH64 else "f32",
                "data": "synthetic (seeded displaced torus)",
                "config": {"workload": f"torus 16384 patches, {W}x{H} primary + {DEPTH} bounce, PBR, 2 point lights",
                           "schedule": args.schedule, "rays_per_frame": rays_per_frame,
                           "primary_rays": W * H, "l2": "flushed (2x L2 written) before every frame",
                           "parallelism": f"replicas x{world}"},
                "e2e": e2e, "gpu_launches": counters["kernel_launches"] * args.steps, "clocks": clk.summary()}
        line.update(extra)
        print(json.dumps(line), flush=True)
    if dist:
        td.destroy_process_group()


if __name__ == "__main__":
    main()
