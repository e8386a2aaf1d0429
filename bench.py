"""Benchmark of the ray--bicubic-patch path on GB300.

Headline workload (one step = one frame): the seeded displaced torus (R=4,
r=1, 128x128 = 16,384 bicubic patches, radial displacement sigma 0.05 on
interior control points), 1920x1080 primary rays plus one mirror bounce,
Cook-Torrance PBR with two point lights and their shadow rays, Bezier clipping
at the reference tolerance 2^-12 in FP32 followed by the FP64 Newton polish
of every hit, on the reference's BVH topology (bit-exact build).

value  = total rays (primary + bounce + shadow) / device time of K frames,
         scene resident in HBM, L2 flushed before every frame.
e2e    = the same through cgs_render_host (pinned host framebuffer, copies inside the
         timed region).
accuracy = max relative t error and hit/miss disagreement of the primary hits
         of a seeded 1% pixel subset against the FP64 oracle (and, beside it,
         against the pure-FP64 GPU search).
Further objects: split_longest (the same frame on the longest-axis BVH
build), precision (2^20 grazing rays), batching (64 scenes in one batch
against 64 plain launches), serving (Poisson request streams through the
continuous-batching server against the plain one-request-per-launch server).
--impl reference: the reference's CPU path (the oracle's restatement of it,
         held bit-identical to the reference's own code by the tests) on all
         host cores, one full frame per step.
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
METRIC = "Mrays/s at <=1e-5 rel-t err vs FP64 (C2 torus 1080p + 1 bounce, PBR)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--schedule", default="wavefront", choices=["wavefront", "plain"])
    ap.add_argument("--precision", default="polish64", choices=["fp32", "polish64", "graze64"])
    ap.add_argument("--split", default="reference", choices=["reference", "longest"],
                    help="BVH split axis of the headline frame")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--quick", action="store_true", help="headline frame only")
    ap.add_argument("--size", default=None, help="WxH of a smaller frame (profiling cases); default 1920x1080")
    ap.add_argument("--no-batching", action="store_true", help="skip the 64-scene batching comparison")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving (Poisson stream) comparison")
    ap.add_argument("--no-precision", action="store_true", help="skip the grazing-ray precision comparison")
    ap.add_argument("--no-tune", action="store_true", help="keep the default engine settings (no autotuner)")
    ap.add_argument("--engine", default=None,
                    help="fixed engine settings for the frame instead of the autotuner's pick, e.g. "
                         "passes=2,collect_threads=256,resolve_threads=128,collect_occupancy=3 (profiling runs)")
    ap.add_argument("--only", default=None, choices=["batching", "serving", "batch-render", "precision"],
                    help="run only this leg and print its JSON object (profiling runs; no bench line); "
                         "batch-render: the batching workload's batched render alone, --warmup + --steps times")
    ap.add_argument("--scene", default="c2",
                    help="frame scene: c2 (the torus, default) or c4:<i> / c5:<i>, the seeded union scene i of "
                         "the batching / serving workloads with its camera (profiling cases)")
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


def onchip_peaks():
    """L1 and L2 load bandwidth of this GPU, measured now with the committed
    probes (cgspline_gb300/membench/membench.cu: 16-byte loads, CUDA events,
    best of three runs).  L1: every CTA re-reads its own 16 KB slice (4 CTAs
    of 256 threads per SM); L2: all CTAs stream a 64 MB buffer through
    ld.global.cg (bypassing L1)."""
    import ctypes as C
    from cgspline_gb300 import build as B
    lib = C.CDLL(B.build_membench())
    lib.cgs_membench.argtypes = [C.c_int, C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int,
                                 C.POINTER(C.c_double)]
    out = {}
    for name, level, nbytes, reps in (("l1", 1, 16 << 10, 4000), ("l2", 2, 64 << 20, 200)):
        best = 0.0
        for _ in range(3):
            v = C.c_double(0.0)
            e = lib.cgs_membench(level, nbytes, 4, 256, reps, 5, C.byref(v))
            if e:
                raise RuntimeError(f"cgs_membench({name}) failed: CUDA error {e}")
            best = max(best, v.value)
        out[name + "_gbs"] = best
    out["how"] = ("membench.cu: L1 = 16 KB slice per CTA re-read 4000x with ld.global.nc.v4 (4 CTAs x 256 threads "
                  "per SM); L2 = 64 MB buffer streamed 200x with ld.global.cg.v4; best of 3, 5 timed launches each")
    return out


def traffic_summary():
    """DRAM bytes per launch of the dominant kernel (k_collect, first pass over
    the frame's primary rays) from the committed ncu capture summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_traffic.json")) as f:
            return json.load(f)
    except Exception:
        return None


# ------------------------------------------------------- replicas (N>1) --
def max_over_ranks(ms: float, td=None, device=None) -> float:
    """The timed region's length as the slowest replica saw it: every rank
    renders its own frames (rays are independent, so the path runs as
    replicas with no data-path collective) and the job lasts as long as its
    slowest rank."""
    if td is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def whole_job_mrays(rays_per_frame: int, steps: int, world: int, total_ms: float) -> float:
    """Whole-job throughput: the rays of all ranks' frames over the slowest rank's time."""
    return rays_per_frame * steps * world / (total_ms * 1e-3) / 1e6


# ----------------------------------------------------------- CPU legs --
def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu model")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def cpu_leg(scene, camera, sample_rows=1):
    """The oracle's restatement of the reference's CPU tracer on every host
    core, over every sample_rows-th row of the frame."""
    import oracle
    o = oracle.OracleScene(scene)
    r = o.render_rows(camera, W, H, 0, sample_rows, depth=DEPTH)
    rays = r["primary"] + r["bounce"] + r["shadow"]
    return {"value": rays / r["seconds"] / 1e6, "unit": "Mrays/s", "cores": r["threads"], "kind": "port",
            "cpu_model": cpu_model(), "nproc": os.cpu_count(),
            "sample": f"every {sample_rows} row(s) of the {W}x{H} frame: {r['primary']} primary + {r['bounce']} "
                      f"bounce + {r['shadow']} shadow rays in {r['seconds']:.2f} s (oracle restatement, "
                      f"{r['threads']} threads, 32x32 tiles)",
            "seconds": r["seconds"], "rays": rays}


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU path on this host's cores, one
    full headline frame per step (the same rows as the cpu_baseline leg).
    The reference's own sources compile only where its tree is present,
    which a GPU machine is not; this arm therefore times the oracle's
    restatement of the reference's CPU tracer, which the tests hold
    bit-identical to the reference build (hits and frames) on these scenes."""
    from cgspline_gb300 import scenes
    if rank != 0:
        return
    scene, cam = scenes.scene_c2(), scenes.camera_c2()
    rows = 1
    for _ in range(args.warmup):
        cpu_leg(scene, cam, 8)
    tot_rays, tot_s, leg = 0, 0.0, None
    for _ in range(args.steps):
        leg = cpu_leg(scene, cam, rows)
        tot_rays += leg["rays"]
        tot_s += leg["seconds"]
    v = tot_rays / tot_s / 1e6
    line = {"metric": METRIC, "value": v, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded displaced torus)",
            "impl": "reference",
            "config": {"workload": f"torus 16384 patches, {W}x{H} primary + {DEPTH} bounce, PBR, 2 point lights, "
                                   f"CPU sample = every {rows} rows"},
            "cpu_baseline": {k: leg[k] for k in ("kind", "cores", "cpu_model", "nproc", "sample")}
                            | {"value": v, "unit": "Mrays/s"},
            "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------- GPU legs --
def tile_order(w, h):
    """Pixel index of each queue position when a w x h image's primary rays
    are queued in 8 x 4 tiles (bands of 4 rows cut into 8-column chunks, the
    order of the render's tiled ray queue)."""
    import numpy as np
    p = np.arange(w * h, dtype=np.int64)
    band = p // (4 * w)
    m = p - band * 4 * w
    hb = np.minimum(4, h - 4 * band)
    c = m // (8 * hb)
    q = m - c * 8 * hb
    cw = np.minimum(8, w - 8 * c)
    return (4 * band + q // cw) * w + 8 * c + q % cw


def timed(torch, stream, flush, fn, reps):
    """Device ms of each of `reps` calls of fn(), L2 flushed before each."""
    e0 = [torch.cuda.Event(enable_timing=True) for _ in range(reps)]
    e1 = [torch.cuda.Event(enable_timing=True) for _ in range(reps)]
    for k in range(reps):
        flush.fill_(float(k))
        e0[k].record(stream)
        fn()
        e1[k].record(stream)
        e1[k].synchronize()
    return [a.elapsed_time(b) for a, b in zip(e0, e1)]


def accuracy_vs_fp64(rt, g, rays, prec, group=None):
    """FP32 (+ polish) hits of `rays` against the pure-FP64 GPU search."""
    import numpy as np
    ref = {k: v.cpu().numpy() for k, v in g.intersect(rays, precision=rt.FP64, group=group).items()}
    a = {k: v.cpu().numpy() for k, v in g.intersect(rays, precision=prec, group=group).items()}
    hit_a, hit_r = a["patch"] >= 0, ref["patch"] >= 0
    both = hit_a & hit_r
    rel = np.abs(a["t"][both] - ref["t"][both]) / ref["t"][both]
    return {"rays": int(rays.shape[1]), "max_rel_t_err": float(rel.max(initial=0.0)),
            "rays_over_1e-5": int((rel > 1e-5).sum()), "hit_miss_disagreement": float((hit_a != hit_r).mean()),
            "patch_disagreement": float((both & (a["patch"] != ref["patch"])).mean()),
            "reference": "pure-FP64 GPU search"}


def accuracy_vs_oracle64(rt, g, rays, prec, scene, method=None):
    """FP32 (+ polish) hits of `rays` against the FP64 oracle (the CPU
    restatement of the reference's search run in double to 1e-9, every root
    polished): the checker of the accuracy bar, untimed."""
    import numpy as np

    import oracle
    ref = oracle.OracleScene(scene).intersect(rays.cpu().numpy(), precision=oracle.FP64)
    kw = {} if method is None else {"method": method}
    a = {k: v.cpu().numpy() for k, v in g.intersect(rays, precision=prec, **kw).items()}
    hit_a, hit_r = a["patch"] >= 0, ref["patch"] >= 0
    both = hit_a & hit_r
    rel = np.abs(a["t"][both] - ref["t"][both]) / ref["t"][both]
    return {"rays": int(rays.shape[1]), "max_rel_t_err": float(rel.max(initial=0.0)),
            "rays_over_1e-5": int((rel > 1e-5).sum()), "hit_miss_disagreement": float((hit_a != hit_r).mean()),
            "patch_disagreement": float((both & (a["patch"] != ref["patch"])).mean()),
            "reference": "FP64 oracle (CPU restatement of the reference's search in double, polished roots)"}


def frame_leg(rt, torch, g, cam, tracer, frame, stream, flush, steps):
    for _ in range(3):
        tracer.render(frame, cam, g, stream)
        torch.cuda.synchronize()
    c = g.counters()
    ms = timed(torch, stream, flush, lambda: tracer.render(frame, cam, g, stream), steps)
    return c, ms


def precision_leg(rt, scenes, torch, dev, g, scene, flush, n=1 << 20):
    """2^20 seeded grazing rays (within 0.5 degrees of the tangent plane at
    random points of the torus): FP32, FP32 + FP64 polish, and the full
    precision form (FP32 + FP64 polish + FP64 fat-line bounds for near-grazing
    candidates) against the pure-FP64 GPU search, with the throughput of each."""
    import numpy as np
    rays = torch.from_numpy(scenes.grazing_rays(scene.surfaces[0], n, seed=3)).to(dev)
    stream = torch.cuda.current_stream()
    out = {"rays": n, "workload": "2^20 grazing rays, torus 16384 patches, closest hit"}
    res = {}
    for name, prec in (("fp64", rt.FP64), ("fp32", rt.FP32), ("fp32_polish64", rt.FP32_POLISH64),
                       ("fp32_graze64", rt.FP32_GRAZE64)):
        g.intersect(rays, precision=prec)
        torch.cuda.synchronize()
        reps = 1 if prec == rt.FP64 else 3
        holder = {}
        ms = timed(torch, stream, flush, lambda: holder.update(r=g.intersect(rays, precision=prec)), reps)
        res[name] = {k: v.cpu().numpy() for k, v in holder["r"].items()}
        out[name] = {"Mrays_s": n / (sum(ms) / reps * 1e-3) / 1e6, "ms": sum(ms) / reps}
    ref = res["fp64"]
    for name in ("fp32", "fp32_polish64", "fp32_graze64"):
        a = res[name]
        both = (a["patch"] >= 0) & (ref["patch"] >= 0)
        rel = np.abs(a["t"][both] - ref["t"][both]) / ref["t"][both]
        out[name].update({"max_rel_t_err": float(rel.max(initial=0.0)),
                          "rays_over_1e-5": int((rel > 1e-5).sum()),
                          "hit_miss_disagreement": float(((a["patch"] >= 0) != (ref["patch"] >= 0)).mean()),
                          "patch_disagreement": float((both & (a["patch"] != ref["patch"])).mean())})
    out["fp64"]["hits"] = int((ref["patch"] >= 0).sum())
    # the checker: every level (and the GPU's own FP64 search) against the FP64 oracle
    import oracle
    host_rays = rays.cpu().numpy()
    o64 = oracle.OracleScene(scene).intersect(host_rays, precision=oracle.FP64)
    for name in ("fp64", "fp32", "fp32_polish64", "fp32_graze64"):
        a = res[name]
        both = (a["patch"] >= 0) & (o64["patch"] >= 0)
        rel = np.abs(a["t"][both] - o64["t"][both]) / o64["t"][both]
        out[name]["vs_oracle64"] = {"max_rel_t_err": float(rel.max(initial=0.0)),
                                    "rays_over_1e-5": int((rel > 1e-5).sum()),
                                    "hit_miss_disagreement": float(((a["patch"] >= 0) != (o64["patch"] >= 0)).mean())}
    return out


def subdivision_leg(rt, torch, g, cam, flush, scene, subset):
    """The two intersectors of the reference on the frame's 2,073,600 primary
    rays (closest hit, FP32, tolerance 2^-12): Bezier clipping
    (doBezierClipping) and subdivision (doSubdivision, the device variant's
    bisection), each timed alone with L2 flushed; their agreement on every
    ray, and each against the FP64 oracle on the 1% subset."""
    import numpy as np
    stream = torch.cuda.current_stream()
    rays = rt.camera_rays(cam, W, H, device=torch.cuda.current_device())
    n = int(rays.shape[1])
    out = {"rays": n, "workload": f"torus 16384 patches, {W}x{H} primary rays, closest hit, FP32"}
    res = {}
    for name, method in (("clip", rt.CLIP), ("subdivision", rt.SUBDIV)):
        g.intersect(rays, method=method)
        torch.cuda.synchronize()
        holder = {}
        ms = timed(torch, stream, flush, lambda: holder.update(r=g.intersect(rays, method=method)), 3)
        res[name] = {k: v.cpu().numpy() for k, v in holder["r"].items()}
        c = g.counters()
        out[name] = {"Mrays_s": n / (sum(ms) / 3 * 1e-3) / 1e6, "ms": sum(ms) / 3,
                     "clip_or_subdivision_iterations_per_ray": c["iterations"] / max(1, c["rays"]),
                     "accuracy": accuracy_vs_oracle64(rt, g, subset, rt.FP32, scene, method=method)}
    a, b = res["clip"], res["subdivision"]
    ha, hb = a["patch"] >= 0, b["patch"] >= 0
    both = ha & hb
    rel = np.abs(a["t"][both] - b["t"][both]) / a["t"][both]
    out["agreement"] = {"hit_miss_disagreement": float((ha != hb).mean()),
                        "patch_disagreement": float((both & (a["patch"] != b["patch"])).mean()),
                        "max_rel_t_diff": float(rel.max(initial=0.0)),
                        "rays_t_diff_over_1e-5": int((rel > 1e-5).sum()),
                        "subdivision_closer_by_1e-5": int((both & (b["t"] < a["t"] * (1 - 1e-5))).sum()),
                        "clip_closer_by_1e-5": int((both & (a["t"] < b["t"] * (1 - 1e-5))).sum())}
    return out


def store_build(rt, scs, dev, split):
    """A resident store of scenes `scs`, built with its phases timed: adding
    the surfaces and objects, the host BVH build (cgs_bvh_build, all host
    cores), upload + perfect-hash build (cgs_hash_build); then the hash build
    alone a second time (the store is resident: keys in, tables out).  The
    hash build's algorithmic bytes are its keys read and its displacement
    and table words written, 4 bytes each, against the HBM roof."""
    import torch
    t0 = time.perf_counter()
    store = rt.GpuScene(scs, device=dev.index or 0, split=split, build=False)
    t1 = time.perf_counter()
    check = rt._capi.check
    check(store.lib.cgs_bvh_build(store.h), "cgs_bvh_build")
    t2 = time.perf_counter()
    check(store.lib.cgs_hash_build(store.h, None), "cgs_hash_build")
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    check(store.lib.cgs_hash_build(store.h, None), "cgs_hash_build")
    torch.cuda.synchronize()
    t4 = time.perf_counter()
    nb = store.nbvh()
    alg = 0
    for k in list(range(store.surfaces)) + [-1 - g for g in range(store.groups)]:
        _, _, n_table, n_disp, n_keys = store.bvh_sizes(k)
        alg += 4 * (n_keys + n_disp + n_table)
    peaks, pk = measured_peaks()
    hash_s = t4 - t3
    timing = {"total_s": t3 - t0, "add_s": t1 - t0, "bvh_build_s": t2 - t1, "upload_and_hash_s": t3 - t2,
              "hash_build_s": hash_s, "bvhs": nb,
              "hash_roofline": {"bound": "hbm", "achieved": alg / hash_s / 1e9, "peak": peaks["hbm_gbs"],
                                "unit": "GB/s", "frac": alg / hash_s / 1e9 / peaks["hbm_gbs"],
                                "algorithmic_bytes": alg, "peak_source": pk,
                                "note": "keys read + displacement and table words written, 4 B each; the build "
                                        "is bound by its round barriers (launches, block syncs), not by bytes"}}
    return store, timing


def batching_leg(rt, scenes, torch, dev, stream, prec, flush, steps=3):
    """64 resident scenes (seeded unions of displaced cube-spheres and tori,
    256..65,536 patches each), one request per scene with 64^2..1024^2 primary
    rays + 1 bounce + shadow rays.  Batched: every request in one
    cgs_render_batch wavefront (replayed from a captured CUDA graph), at the
    engine settings the autotuner picks on this batch for each BVH build (the
    reference build's pick stays in force afterwards).  Plain:
    one k_render_plain launch per request (the reference's per-frame launch
    shape), back to back; both on the reference's BVH topology, and the
    batched path again on the longest-axis build, with the FP32 + FP64-polish
    form and with the full precision form (FP64 fat-line bounds for
    near-grazing candidates added).  The longest-axis legs run on a mirrored
    store (CGS_SPLIT_MIRROR), which exports the reference topology."""
    import numpy as np
    t0 = time.perf_counter()
    scs = [scenes.scene_c4(i) for i in range(64)]
    cams = [scenes.camera_c4(i) for i in range(64)]
    gen_s = time.perf_counter() - t0
    out = {"scenes": 64, "patches": int(sum(s.patch_count for s in scs)),
           "primary_rays": int(sum(side * side for _, side in cams)), "scene_gen_s": gen_s}
    # the longest-axis legs run on a mirrored store (CGS_SPLIT_MIRROR): it traverses the
    # longest-axis build and exports the reference topology, checked here on two BVHs
    out["split_longest_store"] = "CGS_SPLIT_MIRROR"
    ref_export = {}
    for split_name, split in (("reference", rt.SPLIT_REFERENCE), ("longest", rt.SPLIT_MIRROR)):
        store, tm = store_build(rt, scs, dev, split)
        out[f"store_build_s_{split_name}"] = tm["total_s"]
        out[f"store_build_{split_name}"] = tm
        out["footprint_mb"] = store.footprint() / 2 ** 20
        for w in (0, -1):
            b = store.bvh(w)
            if split == rt.SPLIT_REFERENCE:
                ref_export[w] = b
            else:
                out["mirror_export_equals_reference"] = out.get("mirror_export_equals_reference", True) and all(
                    np.array_equal(b[k], ref_export[w][k]) for k in b)
        reqs = [rt.Request.alloc(i, c, side, side, 1, DEPTH, device=dev.index or 0)
                for i, (c, side) in enumerate(cams)]
        # the autotuner picks the engine settings on this batch (outside the timed region)
        t0 = time.perf_counter()
        cfg, tms = rt.autotune(store, reqs, rt.Options(recursion_depth=DEPTH, precision=prec), repeats=3)
        out[f"autotune_{split_name}"] = {"settings": cfg, "ms": tms, "seconds": time.perf_counter() - t0}
        legs = (("batched", rt.WAVEFRONT, prec), ("plain", rt.PLAIN, prec)) if split == rt.SPLIT_REFERENCE else \
            (("batched_split_longest", rt.WAVEFRONT, prec),
             ("batched_split_longest_graze64", rt.WAVEFRONT, rt.FP32_GRAZE64))
        for name, sched, p in legs:
            tr = rt.RayTracer(rt.Options(recursion_depth=DEPTH, precision=p, schedule=sched))
            for _ in range(2):  # the first runs eagerly, the second captures the graph
                tr.render_batch(reqs, store, stream)
                torch.cuda.synchronize()
            c = store.counters()
            ms = timed(torch, stream, flush, lambda: tr.render_batch(reqs, store, stream), steps)
            out[name] = {"value": c["rays"] * steps / (sum(ms) * 1e-3) / 1e6, "unit": "Mrays/s",
                         "ms_per_batch": sum(ms) / steps, "rays": c["rays"], "launches": c["kernel_launches"],
                         "device_errors": c["device_errors"]}
        # accuracy: 1% of every scene's primary rays through per-ray groups, against the FP64 GPU search
        rays, grp = [], []
        for i, (cam, side) in enumerate(cams):
            r = rt.camera_rays(cam, side, side, device=dev.index or 0)
            sub = torch.from_numpy(scenes.random_subset(side * side, 0.01, seed=100 + i)).to(dev)
            rays.append(r[:, sub])
            grp.append(torch.full((sub.numel(),), i, dtype=torch.int32, device=dev))
        rays, grp = torch.cat(rays, 1).contiguous(), torch.cat(grp)
        if split == rt.SPLIT_REFERENCE:
            out["accuracy"] = accuracy_vs_fp64(rt, store, rays, prec, grp)
        else:
            out["accuracy_split_longest"] = accuracy_vs_fp64(rt, store, rays, prec, grp)
            out["accuracy_split_longest_graze64"] = accuracy_vs_fp64(rt, store, rays, rt.FP32_GRAZE64, grp)
        store.close()
    rt.set_engine_config(**out["autotune_reference"]["settings"])
    out["speedup_vs_plain"] = out["batched"]["value"] / out["plain"]["value"]
    out["speedup_vs_plain_split_longest"] = out["batched_split_longest"]["value"] / out["plain"]["value"]
    out["speedup_vs_plain_split_longest_graze64"] = \
        out["batched_split_longest_graze64"]["value"] / out["plain"]["value"]
    out["engine_settings"] = rt.engine_config()
    return out


SERVE_RES = ((256, 256), (512, 512), (1920, 1080), (3840, 2160))
PRECISIONS = {"fp32": lambda rt: rt.FP32, "polish64": lambda rt: rt.FP32_POLISH64,
              "graze64": lambda rt: rt.FP32_GRAZE64}


def serving_stream(n, seed=9):
    """The seeded request mix of the serving workload: scene uniform over the
    32 resident scenes, resolution uniform over SERVE_RES, renders (1..4 spp,
    depth 0..3) and closest-hit ray queries (one ray per pixel) half each."""
    from cgspline_gb300 import scenes
    rng = scenes.SplitMix64(seed)
    u = rng.uniform(5 * n).reshape(n, 5)
    out = []
    for k in range(n):
        kind = "render" if u[k, 0] < 0.5 else "query"
        out.append(dict(kind=kind, scene=int(u[k, 1] * 32) % 32, res=SERVE_RES[int(u[k, 2] * 4) % 4],
                        spp=1 + int(u[k, 3] * 4) % 4, depth=int(u[k, 4] * 4) % 4))
    return out


def serving_leg(rt, scenes, torch, dev, prec, rates=(50, 200, 1000, 2000), nreq=40, slots=2, budget_gb=96):
    """32 resident scenes (1K..1M patches), a Poisson stream of nreq requests
    per rate through the continuous-batching server (reference and
    longest-axis BVH builds, the latter a mirrored store that exports the
    reference topology) and through the plain server (one request per
    launch, one at a time, reference build); p50 / p99 latency from submit to
    completion, and rays/s over the stream.  The engine settings are the ones
    in force (bench.py's batching leg leaves its autotuned pick)."""
    import numpy as np
    t0 = time.perf_counter()
    scs = [scenes.scene_c5(i) for i in range(32)]
    cams = [scenes.camera_c5(i) for i in range(32)]
    gen_s = time.perf_counter() - t0
    stream = serving_stream(nreq)
    out = {"scenes": 32, "patches": int(sum(s.patch_count for s in scs)), "requests_per_rate": nreq,
           "slots": slots, "memory_budget_gb": budget_gb, "scene_gen_s": gen_s, "rates": []}
    stores = {}
    out["split_longest_store"] = "CGS_SPLIT_MIRROR"
    for split_name, split in (("reference", rt.SPLIT_REFERENCE), ("longest", rt.SPLIT_MIRROR)):
        stores[split_name], tm = store_build(rt, scs, dev, split)
        out[f"store_build_s_{split_name}"] = tm["total_s"]
        out[f"store_build_{split_name}"] = tm
    out["footprint_mb"] = stores["reference"].footprint() / 2 ** 20
    # inputs and outputs are allocated before the timed streams
    reqs = []
    for q in stream:
        w, h = q["res"]
        if q["kind"] == "render":
            reqs.append(rt.Request.alloc(q["scene"], cams[q["scene"]], w, h, spp=q["spp"], recursion_depth=q["depth"],
                                         device=dev.index or 0))
        else:
            rays = rt.camera_rays(cams[q["scene"]], w, h, device=dev.index or 0)
            res = (torch.empty((3, w * h), dtype=torch.float32, device=dev),
                   torch.empty((2, w * h), dtype=torch.int32, device=dev))
            reqs.append((q["scene"], rays, res))
    torch.cuda.synchronize()

    def play(server, rate, seed):
        rng = scenes.SplitMix64(seed)
        gaps = -np.log(1.0 - rng.uniform(nreq)) / rate if rate else np.zeros(nreq)
        arrivals = np.cumsum(gaps) - gaps[0]
        r0 = server.stats()["rays_traced"]
        start = time.perf_counter()
        tickets = []
        for k, r in enumerate(reqs):
            while time.perf_counter() - start < arrivals[k]:
                pass
            if isinstance(r, tuple):
                tickets.append(server.submit_query(r[0], r[1], out=r[2])[0])
            else:
                tickets.append(server.submit_render(r))
        infos = [server.wait(t) for t in tickets]
        failed = [i["status"] for i in infos if i["status"] != 0]
        if failed:
            raise RuntimeError(f"serving: {len(failed)} of {len(infos)} requests failed (status {failed[0]})")
        lat = np.array([i["finish_s"] - i["submit_s"] for i in infos]) * 1e3
        span = max(i["finish_s"] for i in infos) - min(i["submit_s"] for i in infos)
        rays = server.stats()["rays_traced"] - r0
        return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "Mrays_s": rays / span / 1e6, "rays": int(rays), "span_s": span}

    opts = rt.Options(recursion_depth=3, precision=prec)
    servers = {"served": rt.Server(stores["reference"], slots=slots, memory_budget=budget_gb << 30, options=opts),
               "served_split_longest": rt.Server(stores["longest"], slots=slots, memory_budget=budget_gb << 30,
                                                 options=opts),
               "plain": rt.Server(stores["reference"], options=rt.Options(recursion_depth=3, precision=prec,
                                                                          schedule=rt.PLAIN))}
    for sv in servers.values():
        play(sv, 0, 1)  # warm-up: slot buffers grow to their working size, graphs get captured
    out["max_batch_samples"] = servers["served"].stats()["max_batch_samples"]
    for k, lam in enumerate(rates):
        out["rates"].append({"lambda": lam} | {name: play(sv, lam, 100 + k) for name, sv in servers.items()})
    sat = {name: play(sv, 0, 7) for name, sv in servers.items()}
    st = servers["served"].stats()
    out["served_stats"] = {k: st[k] for k in ("batches", "chunks", "peak_slot_bytes", "kernel_launches")}
    for sv in servers.values():
        sv.close()
    sat["speedup"] = sat["served"]["Mrays_s"] / sat["plain"]["Mrays_s"]
    sat["speedup_split_longest"] = sat["served_split_longest"]["Mrays_s"] / sat["plain"]["Mrays_s"]
    out["saturation"] = sat
    # accuracy: 1% of 512x512 primary rays of every scene, against the FP64 GPU search
    rays, grp = [], []
    for i, cam in enumerate(cams):
        r = rt.camera_rays(cam, 512, 512, device=dev.index or 0)
        sub = torch.from_numpy(scenes.random_subset(512 * 512, 0.01, seed=200 + i)).to(dev)
        rays.append(r[:, sub])
        grp.append(torch.full((sub.numel(),), i, dtype=torch.int32, device=dev))
    rays, grp = torch.cat(rays, 1).contiguous(), torch.cat(grp)
    out["accuracy_split_longest"] = accuracy_vs_fp64(rt, stores["longest"], rays, prec, grp)
    out["accuracy_split_longest_graze64"] = accuracy_vs_fp64(rt, stores["longest"], rays, rt.FP32_GRAZE64, grp)
    for s in stores.values():
        s.close()
    out["engine_settings"] = rt.engine_config()
    return out


def frame_scene(scenes, name):
    """The frame's scene and camera: the C2 torus, or a union scene of the
    batching (c4:<i>) or serving (c5:<i>) workloads."""
    if name == "c2":
        return scenes.scene_c2(), scenes.camera_c2()
    kind, _, index = name.partition(":")
    if kind == "c4":
        return scenes.scene_c4(int(index)), scenes.camera_c4(int(index))[0]
    if kind == "c5":
        return scenes.scene_c5(int(index)), scenes.camera_c5(int(index))
    raise SystemExit(f"unknown scene {name!r}")


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

    if args.only:
        prec = PRECISIONS[args.precision](rt)
        if args.engine:
            rt.set_engine_config(**{k.strip(): int(v) for k, v in (kv.split("=") for kv in args.engine.split(","))})
        flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
        if args.only == "batch-render":
            scs = [scenes.scene_c4(i) for i in range(64)]
            store = rt.GpuScene(scs, device=local,
                                split=rt.SPLIT_LONGEST if args.split == "longest" else rt.SPLIT_REFERENCE)
            reqs = [rt.Request.alloc(i, c, side, side, 1, DEPTH, device=local)
                    for i, (c, side) in enumerate(scenes.camera_c4(i) for i in range(64))]
            tr = rt.RayTracer(rt.Options(recursion_depth=DEPTH, precision=prec, schedule=rt.WAVEFRONT))
            for _ in range(max(1, args.warmup)):
                tr.render_batch(reqs, store)
                torch.cuda.synchronize()
            ms = timed(torch, torch.cuda.current_stream(), flush, lambda: tr.render_batch(reqs, store), args.steps)
            c = store.counters()
            out = {"Mrays_s": c["rays"] * len(ms) / (sum(ms) * 1e-3) / 1e6, "ms": ms, "counters": c,
                   "engine_settings": rt.engine_config()}
        elif args.only == "precision":
            sc = scenes.scene_c2()
            out = precision_leg(rt, scenes, torch, dev, rt.GpuScene(sc, device=local), sc, flush)
        elif args.only == "batching":
            out = batching_leg(rt, scenes, torch, dev, torch.cuda.current_stream(), prec, flush, steps=args.steps)
        else:
            out = serving_leg(rt, scenes, torch, dev, prec)
        print(json.dumps({args.only: out}), flush=True)
        return

    scene, cam = frame_scene(scenes, args.scene)
    split = rt.SPLIT_LONGEST if args.split == "longest" else rt.SPLIT_REFERENCE
    g = rt.GpuScene(scene, device=local, split=split)
    sched = rt.WAVEFRONT if args.schedule == "wavefront" else rt.PLAIN
    prec = PRECISIONS[args.precision](rt)
    tracer = rt.RayTracer(rt.Options(recursion_depth=DEPTH, precision=prec, schedule=sched))
    frame = rt.Frame(W, H, alignment=32, device=local)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    # the autotuner picks the engine settings on this frame (outside the timed region)
    tuned = None
    if args.engine:
        rt.set_engine_config(**{k.strip(): int(v) for k, v in (kv.split("=") for kv in args.engine.split(","))})
    elif not args.no_tune:
        req = rt.Request(0, cam, W, H, 1, DEPTH, frame.data, None)
        if frame.stride == W:
            cfg, tms = rt.autotune(g, [req], rt.Options(recursion_depth=DEPTH, precision=prec), repeats=3)
            tuned = {"settings": cfg, "ms": tms}
    frame_settings = rt.engine_config()
    # a scene refuses a new render while its previous one is in flight
    # (src/rt/RayTracer.cu:110-116), so frames are issued one at a time and
    # each is timed on the device
    for _ in range(max(3, args.warmup)):
        tracer.render(frame, cam, g, stream)
        torch.cuda.synchronize()
    counters = g.counters()
    if dist:
        td.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = timed(torch, stream, flush, lambda: tracer.render(frame, cam, g, stream), args.steps)
        torch.cuda.synchronize()
    total_ms = max_over_ranks(float(sum(ms)), td if dist else None, dev)
    rays_per_frame = counters["rays"]
    value = whole_job_mrays(rays_per_frame, args.steps, world, total_ms)

    # e2e: the C-ABI host entry point (framebuffer copied to pinned host memory
    # inside the timed region)
    host_fb = torch.empty((H, W), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    tracer.render_host(cam, g, W, H, linear=False, out=(host_fb, None))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        tracer.render_host(cam, g, W, H, linear=False, out=(host_fb, None))
    e2e_s = time.perf_counter() - t0
    e2e = {"value": rays_per_frame * args.steps / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": 44,
           "d2h_bytes_per_step": W * H * 4}

    extra = {}
    if rank == 0:
        c = counters
        nrays, nodes, hashes, cand, iters = c["rays"], c["nodes"], c["hash_lookups"], c["candidates"], c["iterations"]
        peaks, pk = measured_peaks()
        clocks_now = clk.summary()
        mhz = clocks_now["sm_mhz"] or 2070.0
        fp32_peak = SMS * FP32_FLOPS_PER_CLK_SM * mhz * 1e6 / 1e12
        # the dominant kernel, k_collect (the traversal), timed alone through
        # cgs_traverse on the frame's primary rays: the same launch as the
        # frame's first traversal pass.  Algorithmic bytes per ray: 28 in,
        # 64 per inner-node visit, 8 per backtrack (table + displacement).
        prim = rt.camera_rays(cam, W, H, device=local)
        if rt.engine_config()["ray_order"] == 1:
            # the frame queues its primary rays in 8 x 4 pixel tiles: the same order here
            prim = prim[:, torch.from_numpy(tile_order(W, H)).to(prim.device)].contiguous()
        for _ in range(3):
            g.traverse(prim, stream=stream, copy_lengths=False)
        torch.cuda.synchronize()
        kc = g.counters()
        kms = timed(torch, stream, flush, lambda: g.traverse(prim, stream=stream, copy_lengths=False),
                    max(3, args.steps))
        launch_s = sum(kms) / len(kms) / 1e3
        # the same launch at full occupancy (the frame caps the traversal to leave
        # room for the shadow query beside it; batched and served queries do not)
        cap = rt.engine_config()["collect_occupancy"]
        if cap:
            rt.set_engine_config(collect_occupancy=0)
            ums = timed(torch, stream, flush, lambda: g.traverse(prim, stream=stream, copy_lengths=False),
                        max(3, args.steps))
            rt.set_engine_config(collect_occupancy=cap)
            uncapped_s = sum(ums) / len(ums) / 1e3
        else:
            uncapped_s = launch_s
        nprim = int(prim.shape[1])
        k_bytes = 28 * nprim + 64 * kc["nodes"] + 8 * kc["hash_lookups"]
        k_flops = 12 * kc["nodes"]
        achieved = k_bytes / launch_s / 1e9
        tr = traffic_summary()
        onchip = onchip_peaks()
        dram_bytes = tr.get("bytes_per_launch") if tr else None
        # the frame as a whole: a ray (48 B in + out), a 64 B node per
        # inner-node visit, an 8 B hash probe per backtrack, a 256 B patch +
        # 64 B of candidate-list traffic per (ray, patch) search
        alg_bytes = 48 * nrays + 64 * nodes + 8 * hashes + 320 * cand
        alg_flops = 12 * nodes + 296 * cand + 470 * iters + 200 * nrays
        sec_per_frame = total_ms / args.steps / 1e3
        extra["roofline"] = {"bound": "l1", "achieved": achieved, "peak": onchip["l1_gbs"], "unit": "GB/s",
                             "frac": achieved / onchip["l1_gbs"],
                             "traffic": dram_bytes,
                             "peak_source": "measured in this run: " + onchip["how"],
                             "kernel": f"k_collect: traversal, first pass over the frame's {nprim} primary rays",
                             "launch_ms": launch_s * 1e3, "algorithmic_bytes_per_launch": k_bytes,
                             "uncapped": {"launch_ms": uncapped_s * 1e3,
                                          "achieved": k_bytes / uncapped_s / 1e9,
                                          "frac": k_bytes / uncapped_s / 1e9 / onchip["l1_gbs"],
                                          "note": "the same launch with the traversal at full occupancy "
                                                  "(the frame's setting caps it at "
                                                  f"{cap or 'no'} blocks per SM)"},
                             "per_ray": {"nodes": kc["nodes"] / nprim, "hash_lookups": kc["hash_lookups"] / nprim,
                                         "hash_table_reads": kc["hash_table_reads"] / nprim},
                             "note": "the 6.6 MB scene is L2-resident and the node reads are served by L1/L2: "
                                     "ncu shows the L1 data pipe as the busiest unit, so the algorithmic bytes "
                                     "(28 B per ray, 64 B per inner-node visit, 8 B per backtrack) are set against "
                                     "the measured L1 load bandwidth; the other roofs follow",
                             "l2": {"peak": onchip["l2_gbs"], "unit": "GB/s", "frac": achieved / onchip["l2_gbs"],
                                    "note": "algorithmic bytes against the L2 roof (an upper bound on the L2 "
                                            "share: part of them hit in L1)"},
                             "dram": {"achieved": (dram_bytes / launch_s / 1e9) if dram_bytes else None,
                                      "peak": peaks["hbm_gbs"], "unit": "GB/s",
                                      "frac": (dram_bytes / launch_s / 1e9 / peaks["hbm_gbs"]) if dram_bytes
                                      else None, "peak_source": pk},
                             "fp32": {"achieved": k_flops / launch_s / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                                      "frac": k_flops / launch_s / 1e12 / fp32_peak,
                                      "peak_source": f"nominal 152 SM x 256 flop/clk at {mhz:.0f} MHz"},
                             "frame": {"algorithmic_GB_s": alg_bytes / sec_per_frame / 1e9,
                                       "fp32_TFLOP_s": alg_flops / sec_per_frame / 1e12,
                                       "per_ray": {"nodes": nodes / nrays, "hash_lookups": hashes / nrays,
                                                   "hash_table_reads": c["hash_table_reads"] / nrays,
                                                   "candidates": cand / nrays, "clip_iterations": iters / nrays}}}
        # accuracy of the primary hits on a seeded 1% pixel subset
        allr = rt.camera_rays(cam, W, H, device=local)
        sub = torch.from_numpy(scenes.random_subset(W * H, 0.01, seed=77)).to(dev)
        subset = allr[:, sub].contiguous()
        extra["accuracy"] = accuracy_vs_oracle64(rt, g, subset, prec, scene)
        extra["accuracy"]["vs_gpu_fp64"] = accuracy_vs_fp64(rt, g, subset, prec)
    if not args.quick and rank == 0:
        # plain per-frame GPU path (one thread per pixel, the whole chain inline)
        if sched != rt.PLAIN:
            plain = rt.RayTracer(rt.Options(recursion_depth=DEPTH, precision=prec, schedule=rt.PLAIN))
            _, pms = frame_leg(rt, torch, g, cam, plain, frame, stream, flush, 3)
            extra["plain_path"] = {"value": rays_per_frame * 3 / (sum(pms) * 1e-3) / 1e6, "unit": "Mrays/s",
                                   "ms_per_step": sum(pms) / 3}
        # the same frame on the other BVH build: same hits, different node visits
        other = rt.SPLIT_LONGEST if split == rt.SPLIT_REFERENCE else rt.SPLIT_REFERENCE
        g2 = rt.GpuScene(scene, device=local, split=other)
        c2, ms2 = frame_leg(rt, torch, g2, cam, tracer, frame, stream, flush, args.steps)
        ga = {k: v.cpu().numpy() for k, v in g.intersect(subset, precision=prec).items()}
        gb = {k: v.cpu().numpy() for k, v in g2.intersect(subset, precision=prec).items()}
        hit = ga["patch"] >= 0
        name = "split_longest" if other == rt.SPLIT_LONGEST else "split_reference"
        extra[name] = {"value": c2["rays"] * args.steps / (sum(ms2) * 1e-3) / 1e6, "unit": "Mrays/s",
                       "ms_per_step": sum(ms2) / args.steps, "rays_per_frame": c2["rays"],
                       "per_ray_nodes": c2["nodes"] / c2["rays"],
                       "per_ray_hash_lookups": c2["hash_lookups"] / c2["rays"],
                       "per_ray_hash_table_reads": c2["hash_table_reads"] / c2["rays"],
                       "subset_hit_miss_equal": bool(np.array_equal(hit, gb["patch"] >= 0)),
                       "subset_max_rel_t_diff": float(
                           (np.abs(ga["t"][hit] - gb["t"][hit]) / ga["t"][hit]).max(initial=0.0)),
                       "accuracy": accuracy_vs_fp64(rt, g2, subset, prec)}
        g2.close()
        if not args.no_precision:
            extra["precision"] = precision_leg(rt, scenes, torch, dev, g, scene, flush)
        if args.scene == "c2":
            extra["subdivision"] = subdivision_leg(rt, torch, g, cam, flush, scene, subset)
        # the batching leg tunes the engine on its own batch and leaves the
        # reference build's pick in force for the serving leg; without it the
        # served requests run the frame's pick with the traversal uncapped
        rt.set_engine_config(collect_occupancy=0)
        if not args.no_batching:
            extra["batching"] = batching_leg(rt, scenes, torch, dev, stream, prec, flush)
        if not args.no_serving:
            extra["serving"] = serving_leg(rt, scenes, torch, dev, prec)
    if not args.no_cpu and rank == 0 and world == 1:
        extra["cpu_baseline"] = {k: v for k, v in cpu_leg(scene, cam, 1).items() if k not in ("seconds", "rays")}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
                "warmup": max(3, args.warmup), "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32+f64polish" if prec == rt.FP32_POLISH64 else "f32",
                "data": "synthetic (seeded displaced torus)" if args.scene == "c2" else f"synthetic (union scene {args.scene})",
                "config": {"workload": (f"torus 16384 patches, {W}x{H} primary + {DEPTH} bounce, PBR, 2 point lights"
                                        if args.scene == "c2" else
                                        f"union scene {args.scene} ({scene.patch_count} patches), {W}x{H} primary + "
                                        f"{DEPTH} bounce, PBR"),
                           "schedule": args.schedule, "bvh_split": args.split, "rays_per_frame": rays_per_frame,
                           "primary_rays": W * H, "l2": "flushed (2x L2 written) before every frame",
                           "parallelism": f"replicas x{world}"},
                "e2e": e2e, "gpu_launches": counters["kernel_launches"] * args.steps, "clocks": clk.summary(),
                "engine_settings": frame_settings, "autotune": tuned}
        line.update(extra)
        print(json.dumps(line), flush=True)
    if dist:
        td.destroy_process_group()


if __name__ == "__main__":
    main()
