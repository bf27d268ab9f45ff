#!/usr/bin/env python3
"""Benchmark of the GPU path tracer on the 1M-triangle GGX + IBL scene.

Workload (one "step"): a full render of the ~1.03M-triangle scene (512 x 512
height field displaced by 6-octave improved Perlin noise + 64 geodesic
spheres of 8000 triangles, GGX conductors and dielectrics, a seeded 512 x 256
log-normal environment with a 2-degree sun of radiance 5e4) at 1024 x 1024,
64 samples per pixel, max depth 10.  The scene is synthetic and seeded.

* value      - path samples/s with the scene resident in HBM; device time of
               the render measured with CUDA events on the launching stream.
* e2e        - the same metric through the C ABI with host buffers: each step
               copies the scene from pinned host memory to the device
               (slrgpu_scene_reupload), renders and reads the film back.
* roofline   - the dominant kernel's algorithmic bytes per launch (48 B per
               closest-hit query: 32 B ray in, 16 B hit out; 36 B per any-hit
               query; 792 B per shaded bounce) over its average launch time.
* cpu_baseline - the reference renderer (the CPU oracle built from the
               reference's own sources) on a bounded sample of the same scene.

``--workload small`` runs the same scene recipe at a size for profiler
captures (256 x 256 height field, 16 spheres, 512 x 512 pixels, 4 spp); it is
not a benchmark line.

``--workload bpt_box`` renders the box scene with the bidirectional path
tracer (BPTRenderer semantics, 16 vertices per subpath) at 512 x 512 and
16 spp; its CPU baseline is the reference's BPTRenderer.  ``bpt_volumetric``
does the same for VolumetricBPTRenderer on the volumetric box.

``--workload serving`` runs the serving stream (512 requests, Poisson
arrivals at 20/s, 8 scenes of 1k-2M triangles, half with a medium) through
the plain and the batched server, as a burst and at the arrival times, and
prints throughput and p50/p99 latency of both.

``--impl reference`` times the reference renderer alone (rank 0) on a
bounded sample of the same workload.  Under torchrun each rank renders its
own replica (weak scaling; path samples are independent, no collective).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WIDTH = HEIGHT = 1024
SPP = 64
MAX_DEPTH = 10
VOLUMETRIC = False
BPT = False
METRIC = "path samples/s"
WORKLOAD = ("ggx_ibl_1m: 1,034,242-triangle height field (512x512, 6-octave improved Perlin, amplitude 0.2) "
            "+ 64 geodesic spheres (8000 triangles, scale log-uniform 0.05-0.3), GGX conductors/dielectrics "
            "(alpha 0.05-0.6, anisotropy 0-0.8, eta 1.3-1.7), 512x256 log-normal IBL + 2-degree sun (5e4), "
            "1024x1024, 64 spp, max depth 10, seed 0")

# Algorithmic bytes per unit (per closest-hit query, per any-hit query, per
# shaded bounce, per path sample for the film).
BYTES_EXTEND = 48
BYTES_SHADOW = 36
BYTES_SHADE = 792
BYTES_FILM = 256
# Bidirectional tracer: per traced subpath vertex (ray 32 B + state 16 B +
# throughput 64 B in; vertex record 160 B, throughput 64 B, ray and state
# 48 B, previous vertex's reverse densities 8 B out; closest hit 48 B), per
# evaluated connection with a contribution (light vertex 160 B, its
# predecessor 64 B, two density records per MIS term ~64 B, queued
# connection 100 B out) and per shadow ray.
BYTES_BPT_BOUNCE = 440
BYTES_BPT_CONNECT = 390
BYTES_BPT_SHADOW = 164   # queued connection 100 B in, any-hit query, 64 B atomic add out

# DRAM bytes per unit of the surface tracer's kernels, measured by ncu
# (dram__bytes_read.sum + dram__bytes_write.sum, --clock-control none) on the
# first three launches of a kernel in the `small` workload (512 x 512, 4 spp,
# 176k triangles: 1,048,576 paths, ~0.4 GB of path state), divided by the
# units of those launches (slrgpu_context_queue_counts of the same frame).
# The line scales them by the units per launch of the measured workload (the
# full-size run is not captured with more than the launch list).
# kExtendSort, bounces 0-2: 171.8 MB over 1,604,943 closest-hit queries (the
# BVH nodes and triangles that miss L2, the path records of the roulette at
# the hit, the hit records).
EXTEND_DRAM_BYTES_PER_UNIT = 107.0
# kShadeSurf, the first three launches (bounce 0 conductor and dielectric,
# bounce 1 conductor): 258.8 MB over 610,018 shaded paths.
SHADE_DRAM_BYTES_PER_UNIT = 424.3


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons while running."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _ref_frame(ref_holder, desc, spp, seed, threads):
    """One reference render of the workload's frame at `spp` samples per
    pixel; returns render seconds (scene build excluded)."""
    from oracle import oracle as O
    if BPT:   # one BPT render per reference sensor
        ref = ref_holder[0] if ref_holder[0] is not None else O.RefScene(desc)
        ref_holder[0] = None
        _, s = ref.render_bpt(WIDTH, HEIGHT, spp, MAX_DEPTH, seed=seed, threads=threads, volumetric=VOLUMETRIC)
    else:
        if ref_holder[0] is None:
            ref_holder[0] = O.RefScene(desc)
        _, s = ref_holder[0].render(WIDTH, HEIGHT, spp, MAX_DEPTH, seed=seed, threads=threads, volumetric=VOLUMETRIC)
    return s


REFERENCE_BUILD_FLAGS = ("the reference renderer built from its own sources with its release flags (-O3 -DNDEBUG, "
                  "default floating-point contraction) and build-only patches P1-P4, P6-P11 (oracle/build_ref.py)")


def cpu_baseline(desc, threads: int, seconds_cap: float = 40.0):
    """The reference renderer on the workload's own frame: the whole frame
    (all spp) when one pass predicts it within seconds_cap, else as many
    whole passes as fit.  The reference renders a frame as spp passes of one
    sample per pixel over all tiles (PTRenderer.cpp:65-75), so passes are its
    unit of work."""
    from oracle import oracle as O
    O.use_timing_build()
    t0 = time.time()
    holder = [O.RefScene(desc)]
    build_s = time.time() - t0
    t1 = _ref_frame(holder, desc, 1, 0, threads)
    passes = SPP if t1 * SPP <= seconds_cap else max(1, int(seconds_cap / t1))
    secs = _ref_frame(holder, desc, passes, 1, threads)
    total = WIDTH * HEIGHT * passes
    what = f"the whole frame ({WIDTH}x{HEIGHT}, {SPP} spp" if passes == SPP else \
        f"{passes} of the frame's {SPP} passes ({WIDTH}x{HEIGHT}"
    return {"value": total / secs, "unit": METRIC, "cores": threads, "kind": "reference",
            "sample": f"{what}, max depth {MAX_DEPTH}): {total} path samples in {secs:.1f} s with {threads} "
                      f"threads; SBVH build {build_s:.1f} s excluded; {REFERENCE_BUILD_FLAGS}"}


def run_reference(args):
    """The reference arm: each step renders one pass (one sample per pixel,
    all tiles) of the workload's frame on the host cores, the reference's own
    unit of work in its pass loop; the line carries the same config as the
    GPU arm's."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.use_timing_build()
    threads = os.cpu_count() or 1
    desc = WORKLOADS[args.workload]["scene"]()
    holder = [O.RefScene(desc)]
    times = []
    for i in range(args.warmup + args.steps):
        s = _ref_frame(holder, desc, 1, i, threads)
        if i >= args.warmup:
            times.append(s)
    per_step = WIDTH * HEIGHT
    value = per_step * len(times) / sum(times)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural scene)",
            "config": gpu_config(args.workload, args.spp, args.gpus, None),
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "reference",
                             "sample": f"{args.steps} timed passes (one sample per pixel over all tiles, the "
                                       f"reference's pass loop) of the {WIDTH}x{HEIGHT} frame, max depth "
                                       f"{MAX_DEPTH}, {threads} threads; {REFERENCE_BUILD_FLAGS}"},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def _sub_bench(argv):
    """Runs this script with argv in a fresh process; returns its JSON line
    (or the error)."""
    r = subprocess.run([sys.executable, os.path.abspath(__file__), *argv, "--no-extras"], capture_output=True,
                       text=True, timeout=900)
    for ln in reversed(r.stdout.splitlines()):
        if ln.startswith("{"):
            return json.loads(ln)
    return {"error": f"rc {r.returncode}", "stderr_tail": r.stderr[-2000:]}


def gpu_config(workload: str, spp: int, world: int, bvh) -> dict:
    """The config object both arms print for a rendering workload."""
    wl = WORKLOADS[workload]
    cfg = {"workload": wl["text"], "width": wl["width"], "height": wl["height"], "spp": spp,
           "max_depth": wl["depth"], "parallelism": f"replicas x{world}",
           "l2": "path state (GBs) exceeds L2; 1 GiB buffer written between timed steps"}
    return cfg


def serving_requests(n: int, rate: float, seed: int, num_scenes: int):
    """The serving stream: n requests with Poisson arrivals (mean `rate`/s),
    scene uniform over the serving scenes, resolution uniform over
    {64, 128, 256, 512}^2, spp uniform over {4, 16, 64}, max depth 8."""
    import numpy as np
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    t -= t[0]
    res = rng.choice([64, 128, 256, 512], n)
    spp = rng.choice([4, 16, 64], n)
    sc = rng.integers(0, num_scenes, n)
    return [dict(t=float(t[i]), scene=int(sc[i]), res=int(res[i]), spp=int(spp[i]), depth=8, seed=7000 + i)
            for i in range(n)]


def run_serving(args):
    """Serving stream: plain (one request at a time) vs batched (continuous
    batching), open loop at the Poisson arrival times and as a burst."""
    import numpy as np
    from slr_gb300 import api, scenes
    t0 = time.time()
    descs = scenes.serving_scenes(seed=0)
    gen_s = time.time() - t0
    ctx = api.Context(0)
    t0 = time.time()
    scs = [api.Scene(d, context=ctx) for d in descs]
    build_s = time.time() - t0
    reqs = serving_requests(args.requests, 20.0, 0, len(scs))
    grid = lambda r: ((r["res"] + 7) // 8 * 8) ** 2  # noqa: E731
    total_samples = sum(grid(r) * r["spp"] for r in reqs)

    def run(mode, open_loop):
        srv = api.Server(ctx, mode=mode, max_depth=8)
        # warm-up: one small request per scene
        for k, sc in enumerate(scs):
            srv.wait(srv.submit(sc, 64, 64, 1, 8, seed=k, volumetric=descs[k].medium is not None))
        ids, sub = [], []
        start = time.perf_counter()
        for r in reqs:
            if open_loop:
                delay = start + r["t"] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
            sub.append(time.perf_counter())
            ids.append(srv.submit(scs[r["scene"]], r["res"], r["res"], r["spp"], r["depth"], seed=r["seed"],
                                  volumetric=descs[r["scene"]].medium is not None))
        lat, films = [], {}
        for k, rid in enumerate(ids):
            film, info = srv.wait(rid)
            lat.append((info.done_seconds - info.submit_seconds) * 1e3)
            if k % 64 == 0:
                films[k] = film
        end = time.perf_counter()
        st = srv.stats().as_dict()
        srv.close()
        lat = np.array(lat)
        return {"path_samples_per_s": total_samples / (end - start), "seconds": end - start,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "mean_ms": float(lat.mean()), "waves": st["waves"], "kernel_launches": st["kernel_launches"]}, films

    out = {}
    films_by_mode = {}
    for name, mode in (("plain", api.SERVER_PLAIN), ("batched", api.SERVER_BATCHED)):
        burst, films_by_mode[name] = run(mode, open_loop=False)
        poisson, _ = run(mode, open_loop=True)
        out[name] = {"burst": burst, "poisson": poisson}
    same = all(np.array_equal(films_by_mode["plain"][k], films_by_mode["batched"][k]) for k in films_by_mode["plain"])
    line = {"metric": "path samples/s (serving stream, batched)", "value": out["batched"]["burst"]["path_samples_per_s"],
            "unit": "path samples/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded procedural scenes and request stream)",
            "config": {"workload": f"serving: {args.requests} requests, Poisson 20/s, 8 scenes "
                                   f"{[sum(len(m.indices) for m in d.meshes) for d in descs]} triangles "
                                   "(odd ones with a 256^3 fBm medium, volumetric PT), res {64..512}^2, "
                                   "spp {4,16,64}, max depth 8", "hbm_budget_gb": 150,
                       "scene_generation_s": round(gen_s, 1), "scene_build_s": round(build_s, 1)},
            "batched_over_plain_burst": out["batched"]["burst"]["path_samples_per_s"] /
                                        out["plain"]["burst"]["path_samples_per_s"],
            "plain": out["plain"], "batched": out["batched"],
            "films_identical_across_modes": bool(same), "total_path_samples": total_samples}
    print(json.dumps(line))
    return 0


def run_traversal(args):
    """Traversal microbenchmark on the 1M-triangle scene's BVH: 16,777,216
    coherent primary rays (4096x4096 pinhole, pixel centres) and 16,777,216
    incoherent rays (origins uniform over the surface area, directions
    uniform on the sphere, t_max uniform in [0.1, 10]); closest-hit and
    any-hit queries.  Primitive ids and t are checked against the reference
    accelerator on a 65,536-ray sample of each set."""
    import numpy as np
    import torch
    from slr_gb300 import api, scenes
    from oracle import oracle as O
    desc = scenes.heightfield_scene(seed=0)
    scene = api.Scene(desc)
    from slr_gb300 import raysets
    n_side = 4096
    n = n_side * n_side
    coherent = raysets.coherent_rays(desc, n_side)
    incoherent = raysets.incoherent_rays(desc, n, seed=0)
    torch.cuda.synchronize()
    results = {}
    ref = O.RefScene(desc, build=False)
    check_n = 65536
    for name, rays in (("coherent", coherent), ("incoherent", incoherent)):
        for kind in ("closest", "any"):
            anyhit = kind == "any"
            for _ in range(args.warmup):
                scene.trace(rays, anyhit)
            torch.cuda.synchronize()
            times = []
            for _ in range(args.steps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                prim, tt, _, _ = scene.trace(rays, anyhit)
                e1.record()
                torch.cuda.synchronize()
                times.append(e0.elapsed_time(e1) * 1e-3)
            # parity on a sample against the reference accelerator
            sub = rays[:: n // check_n][:check_n].cpu().numpy()
            rp, rt, _, _ = ref.trace(sub, anyhit=anyhit, threads=os.cpu_count())
            gp = prim[:: n // check_n][:check_n].cpu().numpy()
            if anyhit:
                mism = int((gp.astype(bool) != rp).sum())
                t_ok = True
            else:
                gt = tt[:: n // check_n][:check_n].cpu().numpy()
                mism = int((gp.astype(np.uint32) != rp).sum())
                hit = rp != 0xffffffff
                t_ok = bool(np.all(np.abs(gt[hit] - rt[hit]) <= 1e-6 * np.abs(rt[hit])))
            results[f"{name}_{kind}"] = {"rays_per_s": n / (sum(times) / len(times)), "ms": 1e3 * sum(times) / len(times),
                                         "sample_id_mismatches": mism, "sample_t_within_1e-6": t_ok}
    # CPU baseline: the reference accelerator on 1M incoherent closest-hit rays
    sub = incoherent[: 1 << 20].cpu().numpy()
    t0 = time.perf_counter()
    ref.trace(sub, anyhit=False, threads=os.cpu_count())
    cpu_s = time.perf_counter() - t0
    total_rays = 4 * n
    total_s = sum(r["ms"] for r in results.values()) * 1e-3
    line = {"metric": "rays/s", "value": total_rays / total_s, "unit": "rays/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded rays)",
            "config": {"workload": "traversal: 1,034,242-triangle scene, 4-wide BVH from the SBVH; 4096x4096 coherent "
                                   "primary rays and 16,777,216 incoherent rays, closest and any hit",
                       "l2": "rays (512 MB per set) exceed L2"},
            "sets": results,
            "cpu_baseline": {"value": (1 << 20) / cpu_s, "unit": "rays/s", "cores": os.cpu_count(), "kind": "reference",
                             "sample": "1,048,576 incoherent closest-hit rays through the reference SBVH"}}
    print(json.dumps(line))
    return 0


def _workloads():
    from slr_gb300 import scenes
    return {
        "ggx_ibl_1m": dict(width=1024, height=1024, spp=64, depth=10, volumetric=False, text=WORKLOAD,
                           scene=lambda: scenes.heightfield_scene(seed=0)),
        "small": dict(width=512, height=512, spp=4, depth=10, volumetric=False,
                      text="small: 256x256 height field + 16 spheres (freq 12), 256x128 IBL, 512x512, max depth 10",
                      scene=lambda: scenes.heightfield_scene(grid=256, spheres=16, sphere_freq=12, env_size=(256, 128),
                                                             width=512, height=512, seed=0)),
        "box": dict(width=256, height=256, spp=16, depth=8, volumetric=False,
                    text="box_pt: closed box of 10 triangles + 2 rotated boxes, Lambert walls, 0.25x0.25 ceiling "
                         "light of radiance 15, pinhole, 256x256, 16 spp, max depth 8, seed 0",
                    scene=lambda: scenes.box_scene(256, 256)),
        "bpt_box": dict(width=512, height=512, spp=16, depth=16, volumetric=False, bpt=True,
                        text="bpt_box: the box scene (Lambert walls and blocks, 0.25x0.25 ceiling light), "
                             "BPTRenderer, 16 vertices per subpath, 512x512, 16 spp, seed 0",
                        scene=lambda: scenes.box_scene(512, 512)),
        "bpt_volumetric": dict(width=256, height=256, spp=16, depth=16, volumetric=True, bpt=True,
                               text="bpt_volumetric: the volumetric box (256^3 fBm density grid, sigma_t max 20, "
                                    "albedo 0.9, HG g 0.7), VolumetricBPTRenderer, 16 vertices per subpath, "
                                    "256x256, 16 spp",
                               scene=lambda: scenes.medium_box_scene(256, 256, grid=256)),
        "bpt_box_small": dict(width=256, height=256, spp=4, depth=16, volumetric=False, bpt=True,
                              text="bpt_box_small: the bidirectional box workload at 256x256, 4 spp (profiler "
                                   "captures)",
                              scene=lambda: scenes.box_scene(256, 256)),
        "volumetric_small": dict(width=256, height=256, spp=4, depth=32, volumetric=True,
                                 text="volumetric_small: the volumetric box with a 128^3 grid, 256x256, 4 spp, "
                                      "max depth 32 (profiler captures)",
                                 scene=lambda: scenes.medium_box_scene(256, 256, grid=128)),
        "volumetric": dict(width=512, height=512, spp=64, depth=32, volumetric=True,
                           text="volumetric_box: the box filled with a 256^3 fBm density grid (sigma_t max 20, "
                                "albedo 0.9, Henyey-Greenstein g 0.7, 16^3 super voxels), VolumetricPTRenderer, "
                                "512x512, 64 spp, max depth 32",
                           scene=lambda: scenes.medium_box_scene(512, 512, grid=256)),
    }


WORKLOADS = None


def main():
    global WORKLOADS
    WORKLOADS = _workloads()
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--spp", type=int, default=None)
    ap.add_argument("--workload", default="ggx_ibl_1m",
                    choices=["ggx_ibl_1m", "small", "box", "bpt_box", "bpt_volumetric", "bpt_box_small", "volumetric",
                             "volumetric_small", "serving", "traversal"])
    ap.add_argument("--requests", type=int, default=512)
    ap.add_argument("--cpu-seconds", type=float, default=40.0,
                    help="cap on the CPU baseline's render time (whole passes of the frame)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the volumetric and serving sub-benchmarks of the default line")
    args = ap.parse_args()
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "traversal":
        return run_traversal(args)
    global WIDTH, HEIGHT, WORKLOAD, SPP, MAX_DEPTH, VOLUMETRIC, BPT
    wl = WORKLOADS[args.workload]
    WIDTH, HEIGHT, SPP, MAX_DEPTH, VOLUMETRIC, WORKLOAD = (wl["width"], wl["height"], wl["spp"], wl["depth"],
                                                           wl["volumetric"], wl["text"])
    BPT = wl.get("bpt", False)
    if args.workload in ("small", "volumetric_small", "bpt_box_small"):
        args.no_cpu_baseline = True
    if args.spp is None:
        args.spp = SPP
    if args.impl == "reference":
        if args.workload in ("serving", "traversal"):
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no serving loop; its "
                              "traversal is timed by --workload traversal's cpu_baseline"}))
            return 0
        return run_reference(args)

    import numpy as np
    import torch
    from slr_gb300 import api, scenes

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    spp = args.spp
    desc = wl["scene"]()
    ctx = api.Context(local)
    t0 = time.time()
    scene = api.Scene(desc, context=ctx)
    build_s = time.time() - t0
    st = scene.bvh_stats
    seed_base = 1000 * rank
    l2_flush = torch.empty(256 * 1024 * 1024, dtype=torch.float32, device="cuda")

    film_dev = torch.empty((HEIGHT, WIDTH, 16), dtype=torch.float32, device="cuda")
    for i in range(args.warmup):
        scene.render(WIDTH, HEIGHT, spp, MAX_DEPTH, seed=seed_base + i, film=film_dev, volumetric=VOLUMETRIC, bpt=BPT)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    step_ms, launches = [], 0
    kern_ms = [0.0] * 5
    kern_n = [0] * 5
    ext_rays = sh_rays = dropped = 0
    for i in range(args.steps):
        l2_flush.zero_()
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _, rs = scene.render(WIDTH, HEIGHT, spp, MAX_DEPTH, seed=seed_base + 100 + i, film=film_dev,
                             flags=api.FLAG_PROFILE_KERNELS, volumetric=VOLUMETRIC, bpt=BPT)
        e1.record()
        torch.cuda.synchronize()
        barrier()
        step_ms.append(e0.elapsed_time(e1))
        launches += rs.kernel_launches
        for k in range(5):
            kern_ms[k] += rs.kernel_ms[k]
            kern_n[k] += rs.kernel_count[k]
        ext_rays += rs.extension_rays
        sh_rays += rs.shadow_rays
        dropped += rs.dropped_samples
    clk = clocks.stop()
    total_ms = sum(step_ms)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    samples_per_step = WIDTH * HEIGHT * spp
    value = samples_per_step * args.steps * world / (total_ms * 1e-3)

    # End to end through the C ABI with host buffers.
    film_host = torch.empty((HEIGHT, WIDTH, 16), dtype=torch.float32, pin_memory=True)
    film_np = film_host.numpy()
    # one untimed end-to-end step first: it allocates the engine's film
    # buffers for host films, loads the film layout kernel and makes the
    # first copies from the scene's pinned mirrors
    scene.reupload()
    scene.render(WIDTH, HEIGHT, spp, MAX_DEPTH, seed=seed_base + 199, film=film_np, volumetric=VOLUMETRIC, bpt=BPT)
    torch.cuda.synchronize()
    e2e_ms, h2d = [], 0
    for i in range(max(1, args.steps)):
        barrier()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        h2d = scene.reupload()
        scene.render(WIDTH, HEIGHT, spp, MAX_DEPTH, seed=seed_base + 200 + i, film=film_np, volumetric=VOLUMETRIC,
                     bpt=BPT)
        torch.cuda.synchronize()
        e2e_ms.append(1e3 * (time.perf_counter() - t1))
    e2e_total = sum(e2e_ms)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_total], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_total = float(t.item())
    e2e_value = samples_per_step * len(e2e_ms) * world / (e2e_total * 1e-3)

    # Roofline of the dominant kernel.
    names = api.KERNEL_CLASSES
    dom = max(range(5), key=lambda k: kern_ms[k])
    units = {1: (ext_rays, BYTES_EXTEND), 3: (sh_rays, BYTES_SHADOW), 2: (ext_rays, BYTES_SHADE),
             0: (samples_per_step * args.steps, 64), 4: (samples_per_step * args.steps, BYTES_FILM)}
    if BPT:
        units.update({1: (ext_rays, BYTES_BPT_BOUNCE), 2: (sh_rays, BYTES_BPT_CONNECT),
                      3: (sh_rays, BYTES_BPT_SHADOW), 0: (samples_per_step * args.steps, 2 * 160 + 96)})
    peak, peak_kind = load_peaks()

    def class_roofline(k):
        n_units, per_unit = units[k]
        bytes_per_launch = n_units * per_unit / max(1, kern_n[k])
        avg_launch_s = kern_ms[k] * 1e-3 / max(1, kern_n[k])
        achieved = bytes_per_launch / max(1e-12, avg_launch_s) / 1e9
        r = {"bound": "hbm", "kernel": names[k], "achieved": achieved, "peak": peak, "unit": "GB/s",
             "frac": achieved / peak, "peak_source": peak_kind, "traffic": None,
             "bytes_per_unit": per_unit, "units_per_launch": n_units / max(1, kern_n[k]),
             "avg_launch_ms": avg_launch_s * 1e3}
        if not BPT and not VOLUMETRIC and names[k] in ("extend", "shade"):
            dram = EXTEND_DRAM_BYTES_PER_UNIT if names[k] == "extend" else SHADE_DRAM_BYTES_PER_UNIT
            r["traffic"] = dram * n_units / max(1, kern_n[k])
            r["traffic_source"] = (f"ncu DRAM bytes per unit of the class's kernel on the small workload (first three "
                                   f"launches, {dram} B) x units per launch of this run")
        return r

    roofline = class_roofline(dom)
    roofline["kernel_share"] = {names[k]: kern_ms[k] / max(1e-9, sum(kern_ms)) for k in range(5)}
    # the whole wavefront (the survey's sum): 792 B per bounce (which already
    # counts the extension and shadow queries) plus the film's 256 B per
    # path sample, over the summed kernel time of the timed frames
    roofline_wavefront = None
    if not BPT:
        step_bytes = ext_rays * BYTES_SHADE + samples_per_step * args.steps * BYTES_FILM
        step_achieved = step_bytes / max(1e-12, sum(kern_ms) * 1e-3) / 1e9
        roofline_wavefront = {"bound": "hbm", "achieved": step_achieved, "peak": peak, "unit": "GB/s",
                              "frac": step_achieved / peak, "bytes_per_step": step_bytes / max(1, args.steps)}
    if names[dom] == "extend" and not BPT and not VOLUMETRIC:
        roofline["note"] = ("closest-hit BVH walks: bound by the latency of dependent node and triangle loads from L2 "
                            "and by divergent control flow, not by HBM; bytes_per_unit counts only the query's "
                            "compulsory 48 B (ray in, hit out)")
    if VOLUMETRIC and names[dom] == "shadow":
        roofline["note"] = ("the shadow class is dominated by the ratio-tracking transmittance walks, which read the "
                            "density grid from L2 (64 MiB at 256^3; ~91 % L2 hit rate, ~73 % issue activity with 13 "
                            "of 32 lanes active per instruction under ncu): issue- and latency-bound, not HBM-bound; "
                            "bytes_per_unit counts only the shadow ray's 36 B")
    if BPT:   # the bidirectional tracer's kernels behind the classes
        roofline["kernel"] = {0: "kBptInit", 1: "kBptBounce", 2: "kBptConnect", 3: "kBptShadow",
                              4: "kBptAccumulate"}.get(dom, names[dom])
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": gpu_config(args.workload, spp, world, st),
            "scene": {"triangles": st.num_triangles, "sbvh_fragments": st.num_fragments, "bvh_width": st.width,
                      "scene_build_s": round(build_s, 2)},
            "rays_per_s": (ext_rays + sh_rays) * world / (total_ms * 1e-3),
            "dropped_samples": dropped,
            "gpu_launches": launches,
            "roofline": roofline,
            "roofline_shade": class_roofline(2) if not BPT else None,
            "roofline_wavefront": roofline_wavefront,
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": WIDTH * HEIGHT * 16 * 4, "ms_per_step": e2e_total / len(e2e_ms),
                    "steps_ms": [round(x, 3) for x in e2e_ms]},
            "clocks": clk}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(desc, os.cpu_count() or 1, args.cpu_seconds)
    if rank == 0 and world == 1 and args.workload == "ggx_ibl_1m" and not args.no_extras:
        # the other headline configurations, each measured in a process of
        # its own after this line's timed region
        del scene, film_dev, l2_flush
        torch.cuda.empty_cache()
        line["volumetric"] = _sub_bench(["--workload", "volumetric", "--steps", "2", "--warmup", "1",
                                         "--cpu-seconds", "8"])
        line["serving"] = _sub_bench(["--workload", "serving"])
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
